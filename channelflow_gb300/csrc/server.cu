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
// of `slots` fields whose kernels cover all fields at once, with per-field
// nu, dt, base flow and constraint.  The scheduler (pump):
//   1. admits queued requests into free slots, FIFO, skipping requests whose
//      key has no free slot and whose new ensemble would not fit in the HBM
//      budget; a request first runs its start-up steps (DNS::advance's init
//      stepping, channelflow/dns.cpp:156-160) in a one-field staging DNS of
//      its key and then moves into its slot with cfgpu_ensemble_load_slot;
//   2. keeps every ensemble busy on its own stream: when its chunk in flight
//      has completed (an event query, no wait), it processes interval ends and
//      finished requests and enqueues the next chunk, the largest step count
//      that ends no request's interval early (at most max_steps), so small
//      and large ensembles run concurrently without lock-step rounds;
//   3. reads out finished fields, frees their slots and, under memory
//      pressure, drops ensembles without running fields.
// A new ensemble gets as many fields as requests of its key are waiting (at
// most `slots`).  Slots freed by a finished request keep computing on its last
// field until the next request is loaded; fields never interact, so that work
// is wasted, never wrong.  Each result equals the result of the request run
// alone.
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
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
int cfl_async(cfgpu_dns d);
void cfl_collect(cfgpu_dns d, double* out);
int set_priority(cfgpu_dns d, int prio);
cudaStream_t swap_stream(cfgpu_dns d, cudaStream_t s);
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
  bool operator<(const Key& o) const {
    return std::memcmp(this, &o, sizeof(Key)) < 0;
  }
};

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

struct Request {
  long long id = 0;
  cfgpu_grid grid{};
  cfgpu_flags flags{};  // flags.dt follows the request's TimeStep
  Key key{};
  cfgpu_rt::TimeStepH ts;  // N intervals of n steps (fixed-step requests: N = 1, n = nsteps)
  int interval = 0;        // current interval, 1..N
  int left = 0;            // steps left in the current interval
  double cfl_start = 0;    // CFL number at the start of the current interval
  double cfl = 0;          // last CFL number taken
  bool fixed = true;        // fixed-step request: flags.dt as given
  int nsteps = 0, done = 0;
  std::vector<double> u, q;  // FlowField buffers (velocity, pressure)
  int status = ST_QUEUED;
  double t_submit = 0, t_start = 0, t_done = 0;
  int ens = -1, slot = -1;
  std::string err;
};

struct Ens {
  Key key{};
  cfgpu_dns h = nullptr;
  std::vector<long long> slot_req;  // request id per slot, -1 free
  long long bytes = 0;
  int k = 0;                        // steps of the chunk in flight (0: idle)
  bool cfl_pending = false;         // the chunk ends with a CFL pass (some field reaches an interval end)
  cudaEvent_t done = nullptr;       // recorded after the chunk in flight
  int running() const {
    int n = 0;
    for (long long r : slot_req) n += r >= 0;
    return n;
  }
};

}  // namespace

struct cfgpu_server_s {
  cudaStream_t ctrl = nullptr;  // high-priority stream for control work on idle ensembles
  long long max_bytes = 0, used = 0;
  int slots = 8, precision = CFGPU_FP64;
  long long next_id = 1;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::deque<long long> queue;
  std::vector<std::unique_ptr<Ens>> ens;  // null entries are dropped ensembles
  std::map<Key, cfgpu_dns> staging;       // one-field heterogeneous DNS per key
  long long steps_done = 0, field_steps = 0;
  // host-side accounting: seconds in admission (staging), in interval ends (CFL pass, dt changes), chunks
  double t_admit = 0, t_interval = 0;
  long long chunks = 0, dt_changes = 0;
  // finer host-time breakdown (seconds): ensemble/staging creation, set_params, staging runs, slot loads
  double t_create = 0, t_params = 0, t_stage = 0, t_load = 0;
};

namespace {
struct Timer {
  double& acc;
  double t0;
  explicit Timer(double& a) : acc(a), t0(now_s()) {}
  ~Timer() { acc += now_s() - t0; }
};
}  // namespace

namespace {

int make_staging(cfgpu_server_s* s, Request& r, cfgpu_dns* out) {
  auto it = s->staging.find(r.key);
  if (it == s->staging.end()) {
    cfgpu_dns h = nullptr;
    Timer tm(s->t_create);
    SCK(cfgpu_ensemble_create(&r.grid, &r.flags, 1, s->precision, &h));
    s->used += cfgpu_rt::bytes(h);
    // staging work is waited for by the host: schedule it ahead of the ensembles' queued steps
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess) SCK(cfgpu_rt::set_priority(h, greatest));
    it = s->staging.emplace(r.key, h).first;
  }
  *out = it->second;
  return CFGPU_OK;
}

// Control work on an idle ensemble (slot copies, parameter uploads, table builds, reads) goes through the
// server's high-priority stream, ahead of the other ensembles' queued steps.
template <typename F>
int on_ctrl(cfgpu_server_s* s, cfgpu_dns h, const F& f) {
  if (!s->ctrl) return f();
  if (cudaStreamSynchronize(cfgpu_rt::stream(h)) != cudaSuccess) return sfail(CFGPU_ECUDA, "stream sync");
  cudaStream_t old = cfgpu_rt::swap_stream(h, s->ctrl);
  const int st = f();
  cudaStreamSynchronize(s->ctrl);
  cfgpu_rt::swap_stream(h, old);
  return st;
}

int finish(cfgpu_server_s* s, Request& r, cfgpu_dns h, int slot) {
  SCK(on_ctrl(s, h, [&]() { return cfgpu_ensemble_get_field(h, slot, r.u.data(), r.q.data()); }));
  for (double v : r.u)
    if (!std::isfinite(v)) {
      r.status = ST_FAILED;
      r.err = "result is not finite";
      r.t_done = now_s();
      return CFGPU_OK;
    }
  r.status = ST_DONE;
  r.t_done = now_s();
  return CFGPU_OK;
}

int complete_chunk(cfgpu_server_s* s, Ens* e, bool wait, bool* completed);

double slot_cfl(cfgpu_dns h, int slot, int nb) {
  std::vector<double> c(nb);
  if (cfgpu_ensemble_cfl(h, c.data()) != CFGPU_OK) return NAN;
  return c[slot];
}

// Give the staging DNS the request's flags at its current dt and restart its start-up steps.
int stage_restart(cfgpu_server_s* s, cfgpu_dns st, Request& r) {
  Timer tm(s->t_params);
  if (!r.fixed) r.flags.dt = r.ts.value();
  SCK(cfgpu_rt::restart(st));  // first: the start-up tables are then rebuilt with the request's parameters
  return cfgpu_ensemble_set_params(st, 0, &r.flags, nullptr, nullptr);
}

int advance_sync(cfgpu_dns h, int n) {
  SCK(cfgpu_rt::advance_async(h, n));
  if (cudaStreamSynchronize(cfgpu_rt::stream(h)) != cudaSuccess) return sfail(CFGPU_ECUDA, "step failed");
  return CFGPU_OK;
}

// Run the request in the staging DNS (its fields already there) from the start of interval r.interval
// until it is past its start-up steps with steps left in the interval (returns with *done = false) or
// finished (*done = true).  Interval ends inside the start-up phase are handled here as in cfDSI::f.
int stage_run(cfgpu_server_s* s, Request& r, cfgpu_dns st, bool* finished) {
  Timer tm(s->t_stage);
  *finished = false;
  for (;;) {
    r.cfl_start = r.cfl = slot_cfl(st, 0, 1);
    r.left = r.ts.n;
    const int n0 = std::min(cfgpu_rt::startup_steps(st), r.left);
    if (n0 > 0) {
      SCK(advance_sync(st, n0));
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

// Start request r: dt fitted to T, the CFL probe (variable TimeStep), the start-up steps in the staging
// DNS, then into the free slot `slot` of e.
int start_request(cfgpu_server_s* s, Request& r, Ens* e, int slot) {
  cfgpu_dns st = nullptr;
  SCK(make_staging(s, r, &st));
  SCK(stage_restart(s, st, r));
  SCK(cfgpu_ensemble_set_field(st, 0, r.u.data(), r.q.data()));
  r.t_start = now_s();
  r.status = ST_RUNNING;
  if (r.ts.variable) {
    // cfDSI::f: one step to measure the CFL number, adjust, reset_dt, restart from u (q kept)
    SCK(advance_sync(st, 1));
    r.ts.adjust(slot_cfl(st, 0, 1));
    SCK(stage_restart(s, st, r));
    SCK(cfgpu_ensemble_set_field(st, 0, r.u.data(), nullptr));
  }
  r.interval = 1;
  bool finished = false;
  SCK(stage_run(s, r, st, &finished));
  if (finished) return finish(s, r, st, 0);
  bool completed = false;
  SCK(complete_chunk(s, e, true, &completed));  // the new field's steps start after the chunk in flight
  if (e->slot_req[slot] >= 0) {
    // the completed chunk's bookkeeping did not free this slot; find another one (cannot happen: slot was free)
    return sfail(CFGPU_EINVAL, "slot taken");
  }
  {
    Timer tm(s->t_load);
    SCK(on_ctrl(s, e->h, [&]() {
      SCK(cfgpu_ensemble_set_params(e->h, slot, &r.flags, nullptr, nullptr));
      return cfgpu_ensemble_load_slot(e->h, slot, st);
    }));
  }
  e->slot_req[slot] = r.id;
  r.ens = -1;
  for (size_t i = 0; i < s->ens.size(); ++i)
    if (s->ens[i].get() == e) r.ens = (int)i;
  r.slot = slot;
  return CFGPU_OK;
}

// Interval end of the request in slot i of e (its steps of the interval are done).  Returns with the
// slot freed (finished) or holding the request at the start of its next interval.
int interval_end(cfgpu_server_s* s, Ens* e, int i, const std::vector<double>& cfl_now) {
  Request& r = *s->reqs[e->slot_req[i]];
  if (r.interval >= r.ts.N) {
    SCK(finish(s, r, e->h, i));
    e->slot_req[i] = -1;
    return CFGPU_OK;
  }
  if (r.ts.variable && r.ts.adjust(r.cfl_start)) {
    // dt changed: restart the start-up steps at the new dt through the staging DNS, then back into the slot
    s->dt_changes++;
    cfgpu_dns st = nullptr;
    SCK(make_staging(s, r, &st));
    SCK(stage_restart(s, st, r));
    SCK(on_ctrl(s, e->h, [&]() { return cfgpu_rt::store_slot(e->h, i, st); }));
    r.interval++;
    bool finished = false;
    SCK(stage_run(s, r, st, &finished));
    if (finished) {
      SCK(finish(s, r, st, 0));
      e->slot_req[i] = -1;
      return CFGPU_OK;
    }
    Timer tm(s->t_load);
    return on_ctrl(s, e->h, [&]() {
      SCK(cfgpu_ensemble_set_params(e->h, i, &r.flags, nullptr, nullptr));
      return cfgpu_ensemble_load_slot(e->h, i, st);
    });
  }
  r.interval++;
  r.left = r.ts.n;
  r.cfl_start = r.cfl = cfl_now[i];
  return CFGPU_OK;
}

int interval_end(cfgpu_server_s* s, Ens* e, int i, const std::vector<double>& cfl_now);

// The chunk in flight on e has completed (or is waited for when wait): count its steps, handle interval
// ends (CFL numbers of the whole ensemble in one pass) and finished requests.
int complete_chunk(cfgpu_server_s* s, Ens* e, bool wait, bool* completed) {
  *completed = false;
  if (e->k == 0) {
    *completed = true;
    return CFGPU_OK;
  }
  if (wait) {
    if (cudaEventSynchronize(e->done) != cudaSuccess) return sfail(CFGPU_ECUDA, "ensemble step failed");
  } else {
    const cudaError_t q = cudaEventQuery(e->done);
    if (q == cudaErrorNotReady) return CFGPU_OK;
    if (q != cudaSuccess) return sfail(CFGPU_ECUDA, std::string("ensemble step failed: ") + cudaGetErrorString(q));
  }
  *completed = true;
  s->steps_done += e->k;
  bool boundary = false;
  for (long long id : e->slot_req)
    if (id >= 0) {
      Request& r = *s->reqs[id];
      r.done += e->k;
      r.left -= e->k;
      s->field_steps += e->k;
      boundary |= r.left == 0;
    }
  e->k = 0;
  const bool pending = e->cfl_pending;
  e->cfl_pending = false;
  if (!boundary) return CFGPU_OK;
  const double t0 = now_s();
  struct Acc {
    cfgpu_server_s* s;
    double t0;
    ~Acc() { s->t_interval += now_s() - t0; }
  } acc{s, t0};
  std::vector<double> cfl_now(e->slot_req.size(), 0.0);
  if (pending) {
    cfgpu_rt::cfl_collect(e->h, cfl_now.data());  // the CFL pass ran at the end of the chunk
  } else if (cfgpu_ensemble_cfl(e->h, cfl_now.data()) != CFGPU_OK) {
    return sfail(CFGPU_ECUDA, cfgpu_last_error());
  }
  for (int i = 0; i < (int)e->slot_req.size(); ++i)
    if (e->slot_req[i] >= 0 && s->reqs[e->slot_req[i]]->left == 0) SCK(interval_end(s, e, i, cfl_now));
  return CFGPU_OK;
}

Ens* find_slot(cfgpu_server_s* s, const Key& k, int* slot) {
  for (auto& e : s->ens) {
    if (!e || std::memcmp(&e->key, &k, sizeof(Key)) != 0) continue;
    for (int i = 0; i < (int)e->slot_req.size(); ++i)
      if (e->slot_req[i] < 0) {
        *slot = i;
        return e.get();
      }
  }
  return nullptr;
}

// Drop ensembles without running fields (memory pressure).
void drop_idle(cfgpu_server_s* s) {
  for (auto& e : s->ens)
    if (e && e->running() == 0) {
      if (e->k) cudaEventSynchronize(e->done);
      s->used -= e->bytes;
      cfgpu_dns_destroy(e->h);
      if (e->done) cudaEventDestroy(e->done);
      e.reset();
    }
}

int admit_impl(cfgpu_server_s* s);

int admit(cfgpu_server_s* s) {
  const double t0 = now_s();
  const int st = admit_impl(s);
  s->t_admit += now_s() - t0;
  return st;
}

int admit_impl(cfgpu_server_s* s) {
  std::deque<long long> keep;
  bool dropped = false;
  while (!s->queue.empty()) {
    const long long id = s->queue.front();
    s->queue.pop_front();
    Request& r = *s->reqs[id];
    int slot = -1;
    Ens* e = find_slot(s, r.key, &slot);
    if (!e) {
      // Size the new ensemble to the requests of this key waiting now (at most `slots`): an unused slot
      // would still be computed every step.
      int want = 1;
      for (long long q : s->queue)
        if (std::memcmp(&s->reqs[q]->key, &r.key, sizeof(Key)) == 0) want++;
      want = std::min(want, s->slots);
      const long long est = cfgpu_rt::estimate_bytes(r.grid, r.flags, want, s->precision) +
                            (s->staging.count(r.key) ? 0 : cfgpu_rt::estimate_bytes(r.grid, r.flags, 1, s->precision));
      if (s->used + est > s->max_bytes && !dropped) {
        drop_idle(s);
        dropped = true;
      }
      if (s->used + est > s->max_bytes) {
        keep.push_back(id);  // wait for memory; later requests of other keys may still fit
        continue;
      }
      auto ne = std::make_unique<Ens>();
      ne->key = r.key;
      int st;
      {
        Timer tm(s->t_create);
        st = cfgpu_ensemble_create(&r.grid, &r.flags, want, s->precision, &ne->h);
      }
      if (st != CFGPU_OK) {
        r.status = ST_FAILED;
        r.err = cfgpu_last_error();
        continue;
      }
      ne->bytes = cfgpu_rt::bytes(ne->h);
      s->used += ne->bytes;
      if (cudaEventCreateWithFlags(&ne->done, cudaEventDisableTiming) != cudaSuccess) {
        cfgpu_dns_destroy(ne->h);
        s->used -= ne->bytes;
        r.status = ST_FAILED;
        r.err = "cudaEventCreate failed";
        continue;
      }
      ne->slot_req.assign(want, -1);
      slot = 0;
      e = ne.get();
      bool placed = false;
      for (auto& x : s->ens)
        if (!x) {
          x = std::move(ne);
          placed = true;
          break;
        }
      if (!placed) s->ens.push_back(std::move(ne));
    }
    const int st = start_request(s, r, e, slot);
    if (st != CFGPU_OK) {
      r.status = ST_FAILED;
      r.err = cfgpu_last_error();
      if (slot >= 0 && e->slot_req[slot] == r.id) e->slot_req[slot] = -1;
    }
  }
  s->queue = keep;
  // Nothing runs and the next request still does not fit: it never will (fail it rather than wait forever).
  bool running = false;
  for (auto& e : s->ens)
    if (e && e->running()) running = true;
  if (!running && !s->queue.empty()) {
    Request& r = *s->reqs[s->queue.front()];
    s->queue.pop_front();
    r.status = ST_FAILED;
    r.err = "an ensemble for this grid does not fit in the server's memory budget";
    r.t_done = now_s();
  }
  return CFGPU_OK;
}

}  // namespace

extern "C" {

cfgpu_status cfgpu_server_create(long long max_bytes, int slots, int precision, cfgpu_server* out) {
  if (!out || max_bytes <= 0 || slots < 1 || (precision != CFGPU_FP64 && precision != CFGPU_MIXED))
    return sfail(CFGPU_EINVAL, "bad argument");
  auto* s = new cfgpu_server_s();
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess)
    cudaStreamCreateWithPriority(&s->ctrl, cudaStreamNonBlocking, greatest);
  s->max_bytes = max_bytes;
  s->slots = slots;
  s->precision = precision;
  *out = s;
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_submit(cfgpu_server s, const cfgpu_grid* grid, const cfgpu_flags* flags, int nsteps,
                                 const double* u, long long* id) {
  if (!s || !grid || !flags || !u || !id || nsteps < 0) return sfail(CFGPU_EINVAL, "bad argument");
  if (flags->baseflow == CFGPU_ArbitraryBase) return sfail(CFGPU_ENOTSUP, "ArbitraryBase requests are not served");
  if (flags->nonlinearity == CFGPU_Alternating || flags->nonlinearity == CFGPU_Alternating_)
    return sfail(CFGPU_ENOTSUP, "Alternating nonlinearity requests are not served");
  if (flags->dt <= 0) return sfail(CFGPU_EINVAL, "dt must be positive");
  auto r = std::make_unique<Request>();
  r->id = s->next_id++;
  r->grid = *grid;
  r->flags = *flags;
  r->key = make_key(*grid, *flags);
  r->nsteps = nsteps;
  r->ts.n = nsteps;
  r->ts.N = 1;
  r->ts.dT = flags->dt * nsteps;
  r->ts.dt = r->ts.dtmin = r->ts.dtmax = flags->dt;
  const size_t n1 = 2 * (size_t)grid->Ny * grid->Nx * (grid->Nz / 2 + 1);
  r->u.assign(u, u + 3 * n1);
  r->q.assign(n1, 0.0);
  r->t_submit = now_s();
  *id = r->id;
  if (nsteps == 0) {
    r->status = ST_DONE;
    r->t_start = r->t_done = r->t_submit;
  } else {
    s->queue.push_back(r->id);
  }
  s->reqs.emplace(r->id, std::move(r));
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_submit_ft(cfgpu_server s, const cfgpu_grid* grid, const cfgpu_flags* flags,
                                    const cfgpu_timestep* timestep, double T, const double* u, long long* id) {
  if (!s || !grid || !flags || !timestep || !u || !id) return sfail(CFGPU_EINVAL, "bad argument");
  if (T <= 0) return sfail(CFGPU_EINVAL, "T must be positive (f^T(u) with T <= 0 needs no DNS)");
  cfgpu_rt::TimeStepH ts;
  SCK(ts.init(*timestep));
  ts.adjust_for_T(T);
  SCK(cfgpu_server_submit(s, grid, flags, ts.N * ts.n, u, id));
  Request& r = *s->reqs[*id];
  r.ts = ts;
  r.fixed = false;
  r.flags.dt = ts.value();
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_pump(cfgpu_server s, int max_steps, int* active) {
  if (!s || max_steps < 1) return sfail(CFGPU_EINVAL, "bad argument");
  SCK(admit(s));
  for (auto& e : s->ens) {
    if (!e) continue;
    bool completed = false;
    SCK(complete_chunk(s, e.get(), false, &completed));
    if (!completed || !e->running()) continue;
    int k = max_steps;
    for (long long id : e->slot_req)
      if (id >= 0) k = std::min(k, s->reqs[id]->left);
    SCK(cfgpu_rt::advance_async(e->h, k));
    bool boundary = false;
    for (long long id : e->slot_req)
      if (id >= 0 && s->reqs[id]->left == k) boundary = true;
    if (boundary) {
      SCK(cfgpu_rt::cfl_async(e->h));  // CFL numbers at the interval end, read when the chunk completes
      e->cfl_pending = true;
    }
    if (cudaEventRecord(e->done, cfgpu_rt::stream(e->h)) != cudaSuccess) return sfail(CFGPU_ECUDA, "event record");
    e->k = k;
    s->chunks++;
  }
  if (active) {
    int n = (int)s->queue.size();
    for (auto& e : s->ens)
      if (e) n += e->running();
    *active = n;
  }
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_poll(cfgpu_server s, long long id, int* status, double* u, double* times) {
  if (!s || !status) return sfail(CFGPU_EINVAL, "bad argument");
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
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second->status == ST_QUEUED || it->second->status == ST_RUNNING)
    return sfail(CFGPU_EINVAL, "request is unknown or not finished");
  s->reqs.erase(it);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_stats(cfgpu_server s, long long* stats) {
  if (!s || !stats) return sfail(CFGPU_EINVAL, "bad argument");
  int ne = 0, slots = 0, running = 0;
  for (auto& e : s->ens)
    if (e) {
      ne++;
      slots += (int)e->slot_req.size();
      running += e->running();
    }
  stats[0] = s->used;
  stats[1] = ne;
  stats[2] = slots;
  stats[3] = running;
  stats[4] = (long long)s->queue.size();
  stats[5] = s->steps_done;
  stats[6] = s->field_steps;
  stats[7] = s->chunks;
  stats[8] = s->dt_changes;
  stats[9] = (long long)(s->t_admit * 1e6);
  stats[10] = (long long)(s->t_interval * 1e6);
  stats[11] = (long long)(s->t_create * 1e6);
  stats[12] = (long long)(s->t_params * 1e6);
  stats[13] = (long long)(s->t_stage * 1e6);
  stats[14] = (long long)(s->t_load * 1e6);
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_destroy(cfgpu_server s) {
  if (!s) return CFGPU_OK;
  for (auto& e : s->ens)
    if (e) {
      if (e->k) cudaEventSynchronize(e->done);
      cfgpu_dns_destroy(e->h);
      if (e->done) cudaEventDestroy(e->done);
    }
  for (auto& kv : s->staging) cfgpu_dns_destroy(kv.second);
  if (s->ctrl) cudaStreamDestroy(s->ctrl);
  delete s;
  return CFGPU_OK;
}

}  // extern "C"
