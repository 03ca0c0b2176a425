// Request server: continuous batching of DNS integrations and f^T(u)
// evaluations on one GPU.
//
// A request is (grid, flags, time step, initial velocity): either a fixed
// number of steps at flags.dt, or f^T(u) with a TimeStep exactly as cfDSI's
// f(u, T) runs it (channelflow/cfdsi.cpp:705-775): dt fitted to T, with a
// variable TimeStep a one-step CFL probe and then, every dT, the CFL number
// taken at the start of the interval adjusts dt after it (a dt change
// restarts the start-up steps, as DNS::reset_dt does).  Requests whose grid
// and shared flags (schemes, nonlinearity, dealiasing, taucorrection,
// Vsuck, precision) agree form one batch key; every key has field ensembles
// of up to `slots` fields whose kernels cover all fields at once, with
// per-field nu, dt, base flow and constraint.
//
// Threads.  Every ensemble is driven by its own host thread (its worker), so
// that the host-side waits of one ensemble (start-up steps of a new request,
// CFL numbers at an interval end, a dt change, reading a result) never hold
// up the chunks of the others, which keep the GPU busy on their own streams.
// The worker of an ensemble:
//   1. creates its field ensemble and, when it has more than one field, a
//      one-field staging DNS of its key;
//   2. loads the requests assigned to it into free slots: a request first
//      runs its start-up steps (DNS::advance's init stepping,
//      channelflow/dns.cpp:156-160) in the staging DNS, then moves into its
//      slot with cfgpu_ensemble_load_slot (a one-field ensemble runs them
//      itself);
//   3. enqueues a chunk, the largest step count that ends no request's
//      interval early (at most max_steps), with a CFL pass at its end when a
//      request reaches an interval end, waits for it (a blocking event), and
//      handles interval ends, dt changes and finished requests;
//   4. exits when the server drops it (no running fields, memory pressure) or
//      is destroyed.
// cfgpu_server_pump is the admission round: it assigns queued requests FIFO to
// ensembles of their key with free slots, or creates an ensemble sized to the
// requests of that key waiting now (at most `slots`) when its estimated bytes
// fit in the HBM budget (dropping idle ensembles first if they do not), and
// waits briefly for progress.  Slots freed by a finished request keep
// computing on its last field until the next request is loaded; fields never
// interact, so that work is wasted, never wrong.  Each result equals the
// result of the request run alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cfgpu.h"
#include "kernels.h"
#include "timestep.h"

namespace cfgpu_rt {
int advance_async(cfgpu_dns d, int nsteps);
cudaStream_t stream(cfgpu_dns d);
long long bytes(cfgpu_dns d);
int startup_steps(cfgpu_dns d);
int restart(cfgpu_dns d);
int store_slot(cfgpu_dns d, int slot, cfgpu_dns dst);
int reset_version(cfgpu_dns d, int slot);
int cfl_async(cfgpu_dns d);
void cfl_collect(cfgpu_dns d, double* out);
int set_priority(cfgpu_dns d, int prio);
long long estimate_bytes(const cfgpu_grid& grid, const cfgpu_flags& f, int nb, int precision);
}  // namespace cfgpu_rt

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int sfail(int code, const std::string& m) { return cfgpu_record_error(code, m); }

#define SCK(x)                     \
  do {                             \
    int s_ = (x);                  \
    if (s_ != CFGPU_OK) return s_; \
  } while (0)

struct Key {
  int Nx, Ny, Nz;
  double Lx, Lz, a, b, Vsuck;
  int ts, is, nl, da, tc;
};

bool same_key(const Key& a, const Key& b) { return std::memcmp(&a, &b, sizeof(Key)) == 0; }

Key make_key(const cfgpu_grid& g, const cfgpu_flags& f) {
  Key k;
  std::memset(&k, 0, sizeof(k));
  k.Nx = g.Nx; k.Ny = g.Ny; k.Nz = g.Nz;
  k.Lx = g.Lx; k.Lz = g.Lz; k.a = g.a; k.b = g.b;
  k.Vsuck = f.Vsuck;
  k.ts = f.timestepping; k.is = f.initstepping; k.nl = f.nonlinearity; k.da = f.dealiasing; k.tc = f.taucorrection;
  return k;
}

enum { ST_QUEUED = 0, ST_RUNNING = 1, ST_DONE = 2, ST_FAILED = 3 };

// Fields marked (w) belong to the worker of the request's ensemble while the request runs; the others
// are guarded by the server's mutex.
struct Request {
  long long id = 0;
  cfgpu_grid grid{};
  cfgpu_flags flags{};  // (w) flags.dt follows the request's TimeStep
  Key key{};
  cfgpu_rt::TimeStepH ts;  // (w) N intervals of n steps (fixed-step requests: N = 1, n = nsteps)
  int interval = 0;        // (w) current interval, 1..N
  int left = 0;            // (w) steps left in the current interval
  double cfl_start = 0;    // (w) CFL number at the start of the current interval
  double cfl = 0;          // (w) last CFL number taken
  bool fixed = true;       // fixed-step request: flags.dt as given
  int nsteps = 0, done = 0;
  std::vector<double> u, q;  // FlowField buffers (velocity, pressure); (w) until the request is done
  int status = ST_QUEUED;
  double t_submit = 0, t_start = 0, t_done = 0;
  std::string err;
};

struct Ens {
  Key key{};
  cfgpu_grid grid{};
  cfgpu_flags flags{};  // of the request that created the ensemble
  int nb = 1;
  long long bytes = 0;  // reserved device bytes: the estimate until created, then the actual size
  // worker-owned
  cfgpu_dns h = nullptr, stage = nullptr;  // stage: one-field staging DNS (null when nb == 1)
  cudaEvent_t done = nullptr;
  // written by the worker under the server's mutex (the worker reads them without it)
  std::vector<Request*> slot;  // request per slot, null when free
  // guarded by the server's mutex
  std::deque<Request*> pending;  // assigned, not yet loaded
  bool quit = false;             // exit once idle (memory pressure, failure)
  bool abort = false;            // exit after the chunk in flight (server destroyed)
  bool exited = false;
  std::thread th;
  int running() const {
    int n = 0;
    for (Request* r : slot) n += r != nullptr;
    return n;
  }
  int free_slots() const { return nb - running() - (int)pending.size(); }
  bool idle() const { return running() == 0 && pending.empty(); }
  // where a request runs its start-up steps: the staging DNS, or a one-field ensemble itself
  cfgpu_dns startup_dns() const { return stage ? stage : h; }
};

}  // namespace

struct cfgpu_server_s {
  std::mutex mu;
  std::condition_variable cv_work;  // workers: new assignments, quit/abort
  std::condition_variable cv_prog;  // pump: requests finished, workers exited
  int device = 0;
  long long max_bytes = 0, used = 0;
  int slots = 8, precision = CFGPU_FP64;
  std::atomic<int> max_steps{50};
  long long next_id = 1;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::deque<long long> queue;
  std::vector<std::unique_ptr<Ens>> ens;
  long long steps_done = 0, field_steps = 0, chunks = 0, dt_changes = 0, created = 0;
  // host microseconds, summed over the threads: admission (pump), interval ends, creating ensembles and
  // staging DNS, setting staging parameters, running staging steps, loading slots
  std::atomic<long long> us_admit{0}, us_interval{0}, us_create{0}, us_params{0}, us_stage{0}, us_load{0};
};

namespace {

struct Timer {
  std::atomic<long long>& acc;
  double t0;
  explicit Timer(std::atomic<long long>& a) : acc(a), t0(now_s()) {}
  ~Timer() { acc.fetch_add((long long)((now_s() - t0) * 1e6)); }
};

// Wait for the work enqueued so far on h's stream (a blocking-sync event: the worker sleeps).
int wait_stream(Ens* e, cfgpu_dns h) {
  if (cudaEventRecord(e->done, cfgpu_rt::stream(h)) != cudaSuccess) return sfail(CFGPU_ECUDA, "event record");
  const cudaError_t st = cudaEventSynchronize(e->done);
  if (st != cudaSuccess) return sfail(CFGPU_ECUDA, std::string("step failed: ") + cudaGetErrorString(st));
  return CFGPU_OK;
}

int advance_sync(Ens* e, cfgpu_dns h, int n) {
  SCK(cfgpu_rt::advance_async(h, n));
  return wait_stream(e, h);
}

double slot_cfl(cfgpu_dns h, int slot, int nb) {
  std::vector<double> c(nb);
  if (cfgpu_ensemble_cfl(h, c.data()) != CFGPU_OK) return NAN;
  return c[slot];
}

// Mark r done (failed when its field is not finite) and free slot ens_slot; field `slot` of h holds its
// final state.
int finish(cfgpu_server_s* s, Ens* e, Request& r, cfgpu_dns h, int slot, int ens_slot) {
  SCK(cfgpu_ensemble_get_field(h, slot, r.u.data(), r.q.data()));
  bool finite = true;
  for (double v : r.u) finite &= std::isfinite(v);
  std::lock_guard<std::mutex> lk(s->mu);
  r.status = finite ? ST_DONE : ST_FAILED;
  if (!finite) r.err = "result is not finite";
  r.t_done = now_s();
  e->slot[ens_slot] = nullptr;
  s->cv_prog.notify_all();
  return CFGPU_OK;
}

void fail_request(cfgpu_server_s* s, Ens* e, Request& r, int ens_slot, const std::string& why) {
  std::lock_guard<std::mutex> lk(s->mu);
  r.status = ST_FAILED;
  r.err = why;
  r.t_done = now_s();
  if (e->slot[ens_slot] == &r) e->slot[ens_slot] = nullptr;
  s->cv_prog.notify_all();
}

// Fail every request of e (assigned or running) with `why`; e exits.
void fail_all(cfgpu_server_s* s, Ens* e, const std::string& why) {
  std::lock_guard<std::mutex> lk(s->mu);
  const double t = now_s();
  auto fail1 = [&](Request* r) {
    r->status = ST_FAILED;
    r->err = why;
    r->t_done = t;
  };
  for (Request*& r : e->slot)
    if (r) {
      fail1(r);
      r = nullptr;
    }
  for (Request* r : e->pending) fail1(r);
  e->pending.clear();
  e->quit = true;
  s->cv_prog.notify_all();
}

// Give the staging DNS the request's flags at its current dt and restart its start-up steps.
int stage_restart(cfgpu_server_s* s, cfgpu_dns st, Request& r) {
  Timer tm(s->us_params);
  if (!r.fixed) r.flags.dt = r.ts.value();
  SCK(cfgpu_rt::restart(st));  // first: the start-up tables are then rebuilt with the request's parameters
  return cfgpu_ensemble_set_params(st, 0, &r.flags, nullptr, nullptr);
}

// Run the request in the staging DNS (its fields already there) from the start of interval r.interval
// until it is past its start-up steps with steps left in the interval (returns with *finished = false)
// or finished (*finished = true).  Interval ends inside the start-up phase are handled here as in
// cfDSI::f.
int stage_run(cfgpu_server_s* s, Ens* e, Request& r, bool* finished) {
  Timer tm(s->us_stage);
  cfgpu_dns st = e->startup_dns();
  *finished = false;
  for (;;) {
    r.cfl_start = r.cfl = slot_cfl(st, 0, 1);
    r.left = r.ts.n;
    const int n0 = std::min(cfgpu_rt::startup_steps(st), r.left);
    if (n0 > 0) {
      SCK(advance_sync(e, st, n0));
      r.left -= n0;
      r.done += n0;
    }
    if (r.left > 0) return CFGPU_OK;
    if (r.interval >= r.ts.N) {
      *finished = true;
      return CFGPU_OK;
    }
    if (r.ts.variable && r.ts.adjust(r.cfl_start)) SCK(stage_restart(s, st, r));
    r.interval++;
  }
}

// Move the request, past its start-up steps in the staging DNS, into slot i of the ensemble.
int load_into(cfgpu_server_s* s, Ens* e, Request& r, int i) {
  if (!e->stage) return CFGPU_OK;  // ran in place
  Timer tm(s->us_load);
  SCK(cfgpu_ensemble_set_params(e->h, i, &r.flags, nullptr, nullptr));
  return cfgpu_ensemble_load_slot(e->h, i, e->stage);
}

// Start request r (in slot i, no chunk in flight): dt fitted to T, the CFL probe (variable TimeStep),
// the start-up steps in the staging DNS, then into the slot.
int start_request(cfgpu_server_s* s, Ens* e, Request& r, int i) {
  cfgpu_dns st = e->startup_dns();
  SCK(stage_restart(s, st, r));
  SCK(cfgpu_rt::reset_version(st, 0));  // as a DNS built for this request: its FP32 constants from version 0
  SCK(cfgpu_ensemble_set_field(st, 0, r.u.data(), r.q.data()));
  if (r.ts.variable) {
    // cfDSI::f: one step to measure the CFL number, adjust, reset_dt, restart from u (q kept)
    SCK(advance_sync(e, st, 1));
    r.ts.adjust(slot_cfl(st, 0, 1));
    SCK(stage_restart(s, st, r));
    SCK(cfgpu_ensemble_set_field(st, 0, r.u.data(), nullptr));
  }
  r.interval = 1;
  bool finished = false;
  SCK(stage_run(s, e, r, &finished));
  if (finished) return finish(s, e, r, st, 0, i);
  return load_into(s, e, r, i);
}

// Interval end of the request in slot i (its steps of the interval are done).  Returns with the slot
// freed (finished) or holding the request at the start of its next interval.
int interval_end(cfgpu_server_s* s, Ens* e, int i, double cfl_now) {
  Request& r = *e->slot[i];
  if (r.interval >= r.ts.N) return finish(s, e, r, e->h, i, i);
  if (r.ts.variable && r.ts.adjust(r.cfl_start)) {
    // dt changed: restart the start-up steps at the new dt through the staging DNS, then back into the slot
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->dt_changes++;
    }
    SCK(stage_restart(s, e->startup_dns(), r));
    if (e->stage) SCK(cfgpu_rt::store_slot(e->h, i, e->stage));
    r.interval++;
    bool finished = false;
    SCK(stage_run(s, e, r, &finished));
    if (finished) return finish(s, e, r, e->startup_dns(), 0, i);
    return load_into(s, e, r, i);
  }
  r.interval++;
  r.left = r.ts.n;
  r.cfl_start = r.cfl = cfl_now;
  return CFGPU_OK;
}

int create_handles(cfgpu_server_s* s, Ens* e) {
  Timer tm(s->us_create);
  SCK(cfgpu_ensemble_create(&e->grid, &e->flags, e->nb, s->precision, &e->h));
  if (e->nb > 1) {
    SCK(cfgpu_ensemble_create(&e->grid, &e->flags, 1, s->precision, &e->stage));
    // staging work is waited for by its worker: schedule it ahead of the ensembles' queued steps
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess)
      SCK(cfgpu_rt::set_priority(e->stage, greatest));
  }
  if (cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess)
    return sfail(CFGPU_ECUDA, "cudaEventCreate failed");
  return CFGPU_OK;
}

void release_handles(Ens* e) {
  if (e->h) cfgpu_dns_destroy(e->h);
  if (e->stage) cfgpu_dns_destroy(e->stage);
  if (e->done) cudaEventDestroy(e->done);
  e->h = e->stage = nullptr;
  e->done = nullptr;
}

void worker(cfgpu_server_s* s, Ens* e) {
  cudaSetDevice(s->device);
  int st = create_handles(s, e);
  if (st == CFGPU_OK) {
    std::lock_guard<std::mutex> lk(s->mu);
    const long long actual = cfgpu_rt::bytes(e->h) + (e->stage ? cfgpu_rt::bytes(e->stage) : 0);
    s->used += actual - e->bytes;
    e->bytes = actual;
    s->created++;
  } else {
    fail_all(s, e, cfgpu_last_error());
  }
  std::vector<std::pair<Request*, int>> starting;
  std::vector<double> cfl_now(e->nb, 0.0);
  while (st == CFGPU_OK) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return e->abort || e->quit || !e->pending.empty() || e->running() > 0; });
      if (e->abort || (e->quit && e->idle())) break;
      const double t = now_s();
      for (int i = 0; i < e->nb && !e->pending.empty(); ++i)
        if (!e->slot[i]) {
          Request* r = e->pending.front();
          e->pending.pop_front();
          e->slot[i] = r;
          r->status = ST_RUNNING;
          r->t_start = t;
          starting.push_back({r, i});
        }
    }
    for (auto& ri : starting)
      if (start_request(s, e, *ri.first, ri.second) != CFGPU_OK)
        fail_request(s, e, *ri.first, ri.second, cfgpu_last_error());
    starting.clear();
    // next chunk: the largest step count that ends no request's interval early
    int k = s->max_steps.load();
    bool any = false;
    for (Request* r : e->slot)
      if (r) {
        any = true;
        k = std::min(k, r->left);
      }
    if (!any) continue;
    bool boundary = false;
    for (Request* r : e->slot) boundary |= r && r->left == k;
    if ((st = cfgpu_rt::advance_async(e->h, k)) == CFGPU_OK && boundary) st = cfgpu_rt::cfl_async(e->h);
    if (st == CFGPU_OK) st = wait_stream(e, e->h);
    if (st != CFGPU_OK) {
      fail_all(s, e, cfgpu_last_error());
      break;
    }
    bool abort = false;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->chunks++;
      s->steps_done += k;
      for (Request* r : e->slot)
        if (r) {
          r->done += k;
          r->left -= k;
          s->field_steps += k;
        }
      abort = e->abort;
    }
    if (abort) break;
    if (!boundary) continue;
    Timer tm(s->us_interval);
    cfgpu_rt::cfl_collect(e->h, cfl_now.data());  // the CFL pass ran at the end of the chunk
    for (int i = 0; i < e->nb; ++i) {
      Request* r = e->slot[i];
      if (r && r->left == 0 && interval_end(s, e, i, cfl_now[i]) != CFGPU_OK)
        fail_request(s, e, *r, i, cfgpu_last_error());
    }
  }
  release_handles(e);
  std::lock_guard<std::mutex> lk(s->mu);
  s->used -= e->bytes;
  e->exited = true;
  s->cv_prog.notify_all();
}

// Join and remove the ensembles whose workers have exited (the caller holds the lock; an exited worker
// no longer takes it).
void reap(cfgpu_server_s* s) {
  for (auto& e : s->ens)
    if (e && e->exited) {
      if (e->th.joinable()) e->th.join();
      e.reset();
    }
  s->ens.erase(std::remove(s->ens.begin(), s->ens.end(), nullptr), s->ens.end());
}

// Memory pressure: stop the ensembles without running or assigned fields and wait until their memory
// is back.
void drop_idle(cfgpu_server_s* s, std::unique_lock<std::mutex>& lk) {
  bool any = false;
  for (auto& e : s->ens)
    if (e && !e->exited && e->idle()) {
      e->quit = true;
      any = true;
    }
  if (!any) return;
  s->cv_work.notify_all();
  s->cv_prog.wait(lk, [&] {
    for (auto& e : s->ens)
      if (e && e->quit && !e->exited) return false;
    return true;
  });
  reap(s);
}

void admit(cfgpu_server_s* s, std::unique_lock<std::mutex>& lk) {
  Timer tm(s->us_admit);
  std::deque<long long> keep;
  bool dropped = false, notify = false;
  while (!s->queue.empty()) {
    const long long id = s->queue.front();
    s->queue.pop_front();
    Request* r = s->reqs[id].get();
    Ens* e = nullptr;
    for (auto& x : s->ens)
      if (x && !x->quit && !x->exited && same_key(x->key, r->key) && x->free_slots() > 0) {
        e = x.get();
        break;
      }
    if (e) {
      e->pending.push_back(r);
      notify = true;
      continue;
    }
    // Size the new ensemble to the requests of this key waiting now (at most `slots`): an unused slot
    // would still be computed every step.
    int want = 1;
    for (long long q : s->queue)
      if (same_key(s->reqs[q]->key, r->key)) want++;
    want = std::min(want, s->slots);
    const long long est = cfgpu_rt::estimate_bytes(r->grid, r->flags, want, s->precision) +
                          (want > 1 ? cfgpu_rt::estimate_bytes(r->grid, r->flags, 1, s->precision) : 0);
    if (s->used + est > s->max_bytes && !dropped) {
      drop_idle(s, lk);
      dropped = true;
    }
    if (s->used + est > s->max_bytes) {
      keep.push_back(id);  // wait for memory; later requests of other keys may still fit
      continue;
    }
    auto ne = std::make_unique<Ens>();
    ne->key = r->key;
    ne->grid = r->grid;
    ne->flags = r->flags;
    ne->nb = want;
    ne->bytes = est;
    ne->slot.assign(want, nullptr);
    ne->pending.push_back(r);
    s->used += est;
    Ens* raw = ne.get();
    s->ens.push_back(std::move(ne));
    raw->th = std::thread(worker, s, raw);
  }
  s->queue = keep;
  if (notify) s->cv_work.notify_all();
  // Nothing runs and the next request still does not fit: it never will (fail it rather than wait forever).
  bool busy = false;
  for (auto& e : s->ens)
    if (e && !e->exited && !e->idle()) busy = true;
  if (!busy && !s->queue.empty()) {
    Request& r = *s->reqs[s->queue.front()];
    s->queue.pop_front();
    r.status = ST_FAILED;
    r.err = "an ensemble for this grid does not fit in the server's memory budget";
    r.t_done = now_s();
  }
}

int count_active(cfgpu_server_s* s) {
  int n = (int)s->queue.size();
  for (auto& e : s->ens)
    if (e && !e->exited) n += e->running() + (int)e->pending.size();
  return n;
}

int check_request(const cfgpu_grid* grid, const cfgpu_flags* flags, const double* u, long long* id) {
  if (!grid || !flags || !u || !id) return sfail(CFGPU_EINVAL, "bad argument");
  if (flags->baseflow == CFGPU_ArbitraryBase) return sfail(CFGPU_ENOTSUP, "ArbitraryBase requests are not served");
  if (flags->nonlinearity == CFGPU_Alternating || flags->nonlinearity == CFGPU_Alternating_)
    return sfail(CFGPU_ENOTSUP, "Alternating nonlinearity requests are not served");
  if (flags->dt <= 0) return sfail(CFGPU_EINVAL, "dt must be positive");
  return CFGPU_OK;
}

std::unique_ptr<Request> new_request(const cfgpu_grid* grid, const cfgpu_flags* flags, const double* u) {
  auto r = std::make_unique<Request>();
  r->grid = *grid;
  r->flags = *flags;
  r->key = make_key(*grid, *flags);
  const size_t n1 = 2 * (size_t)grid->Ny * grid->Nx * (grid->Nz / 2 + 1);
  r->u.assign(u, u + 3 * n1);
  r->q.assign(n1, 0.0);
  r->t_submit = now_s();
  return r;
}

void enqueue(cfgpu_server_s* s, std::unique_ptr<Request> r, long long* id) {
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  *id = r->id;
  if (r->nsteps == 0) {
    r->status = ST_DONE;
    r->t_start = r->t_done = r->t_submit;
  } else {
    s->queue.push_back(r->id);
  }
  s->reqs.emplace(r->id, std::move(r));
}

}  // namespace

extern "C" {

cfgpu_status cfgpu_server_create(long long max_bytes, int slots, int precision, cfgpu_server* out) {
  if (!out || max_bytes <= 0 || slots < 1 || (precision != CFGPU_FP64 && precision != CFGPU_MIXED))
    return sfail(CFGPU_EINVAL, "bad argument");
  auto* s = new cfgpu_server_s();
  cudaGetDevice(&s->device);
  s->max_bytes = max_bytes;
  s->slots = slots;
  s->precision = precision;
  *out = s;
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_submit(cfgpu_server s, const cfgpu_grid* grid, const cfgpu_flags* flags, int nsteps,
                                 const double* u, long long* id) {
  if (!s || nsteps < 0) return sfail(CFGPU_EINVAL, "bad argument");
  SCK(check_request(grid, flags, u, id));
  auto r = new_request(grid, flags, u);
  r->nsteps = nsteps;
  r->ts.n = nsteps;
  r->ts.N = 1;
  r->ts.dT = flags->dt * nsteps;
  r->ts.dt = r->ts.dtmin = r->ts.dtmax = flags->dt;
  enqueue(s, std::move(r), id);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_submit_ft(cfgpu_server s, const cfgpu_grid* grid, const cfgpu_flags* flags,
                                    const cfgpu_timestep* timestep, double T, const double* u, long long* id) {
  if (!s || !timestep) return sfail(CFGPU_EINVAL, "bad argument");
  SCK(check_request(grid, flags, u, id));
  if (T <= 0) return sfail(CFGPU_EINVAL, "T must be positive (f^T(u) with T <= 0 needs no DNS)");
  cfgpu_rt::TimeStepH ts;
  SCK(ts.init(*timestep));
  ts.adjust_for_T(T);
  auto r = new_request(grid, flags, u);
  r->nsteps = ts.N * ts.n;
  r->ts = ts;
  r->fixed = false;
  r->flags.dt = ts.value();
  enqueue(s, std::move(r), id);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_pump(cfgpu_server s, int max_steps, int* active) {
  if (!s || max_steps < 1) return sfail(CFGPU_EINVAL, "bad argument");
  s->max_steps.store(max_steps);
  std::unique_lock<std::mutex> lk(s->mu);
  reap(s);
  admit(s, lk);
  int n = count_active(s);
  if (n > 0) {
    // a scheduling round: wait a little for a request to finish or a worker to exit
    s->cv_prog.wait_for(lk, std::chrono::milliseconds(2));
    n = count_active(s);
  }
  if (active) *active = n;
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_poll(cfgpu_server s, long long id, int* status, double* u, double* times) {
  if (!s || !status) return sfail(CFGPU_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return sfail(CFGPU_EINVAL, "unknown request id");
  const Request& r = *it->second;
  *status = r.status;
  if (r.status == ST_DONE && u) memcpy(u, r.u.data(), r.u.size() * sizeof(double));
  if (times) {
    times[0] = r.t_submit;
    times[1] = r.t_start;
    times[2] = r.t_done;
  }
  if (r.status == ST_FAILED) return sfail(CFGPU_ENONFINITE, "request failed: " + r.err);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_release(cfgpu_server s, long long id) {
  if (!s) return sfail(CFGPU_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second->status == ST_QUEUED || it->second->status == ST_RUNNING)
    return sfail(CFGPU_EINVAL, "request is unknown or not finished");
  s->reqs.erase(it);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_stats(cfgpu_server s, long long* stats) {
  if (!s || !stats) return sfail(CFGPU_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  int slots = 0, running = 0;
  for (auto& e : s->ens)
    if (e && !e->exited) {
      slots += e->nb;
      running += e->running();
    }
  stats[0] = s->used;
  stats[1] = s->created;
  stats[2] = slots;
  stats[3] = running;
  stats[4] = (long long)s->queue.size();
  stats[5] = s->steps_done;
  stats[6] = s->field_steps;
  stats[7] = s->chunks;
  stats[8] = s->dt_changes;
  stats[9] = s->us_admit.load();
  stats[10] = s->us_interval.load();
  stats[11] = s->us_create.load();
  stats[12] = s->us_params.load();
  stats[13] = s->us_stage.load();
  stats[14] = s->us_load.load();
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_destroy(cfgpu_server s) {
  if (!s) return CFGPU_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& e : s->ens)
      if (e) e->abort = true;
    s->cv_work.notify_all();
  }
  for (auto& e : s->ens)
    if (e && e->th.joinable()) e->th.join();
  delete s;
  return CFGPU_OK;
}

}  // extern "C"
