// Request server: continuous batching of DNS integrations and f^T(u)
// evaluations on one GPU.
//
// A request is (grid, flags, number of steps, initial velocity).  Requests
// whose grid and shared flags (dt, schemes, nonlinearity, dealiasing,
// taucorrection, Vsuck, precision) agree form one batch key; every key has
// field ensembles of `slots` fields whose kernels cover all fields at once,
// with per-field nu, base flow and constraint.  The scheduler (pump):
//   1. admits queued requests into free slots, FIFO, skipping requests whose
//      key has no free slot and whose new ensemble would not fit in the HBM
//      budget; a request first runs its start-up steps (DNS::advance's init
//      stepping, channelflow/dns.cpp:156-160) in a one-field staging DNS of
//      its key and then moves into its slot with cfgpu_ensemble_load_slot;
//   2. advances every ensemble with running fields by the largest step count
//      that ends no request early, all ensembles enqueued on their own
//      streams before any is waited for, so their kernels overlap;
//   3. reads out finished fields, frees their slots and, under memory
//      pressure, drops ensembles without running fields.
// Slots freed by a finished request keep computing on its last field until
// the next request is loaded; fields never interact, so that work is wasted,
// never wrong.  Each result equals the result of the request run alone.
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

namespace cfgpu_rt {
int advance_async(cfgpu_dns d, int nsteps);
cudaStream_t stream(cfgpu_dns d);
long long bytes(cfgpu_dns d);
int startup_steps(cfgpu_dns d);
int restart(cfgpu_dns d);
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
  double Lx, Lz, a, b, dt, Vsuck;
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
  k.dt = f.dt; k.Vsuck = f.Vsuck;
  k.ts = f.timestepping; k.is = f.initstepping; k.nl = f.nonlinearity; k.da = f.dealiasing; k.tc = f.taucorrection;
  return k;
}

enum { ST_QUEUED = 0, ST_RUNNING = 1, ST_DONE = 2, ST_FAILED = 3 };

struct Request {
  long long id = 0;
  cfgpu_grid grid{};
  cfgpu_flags flags{};
  Key key{};
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
  int k = 0;  // steps enqueued this round
  int running() const {
    int n = 0;
    for (long long r : slot_req) n += r >= 0;
    return n;
  }
};

}  // namespace

struct cfgpu_server_s {
  long long max_bytes = 0, used = 0;
  int slots = 8, precision = CFGPU_FP64;
  long long next_id = 1;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::deque<long long> queue;
  std::vector<std::unique_ptr<Ens>> ens;  // null entries are dropped ensembles
  std::map<Key, cfgpu_dns> staging;       // one-field heterogeneous DNS per key
  long long steps_done = 0, field_steps = 0;
};

namespace {

int make_staging(cfgpu_server_s* s, Request& r, cfgpu_dns* out) {
  auto it = s->staging.find(r.key);
  if (it == s->staging.end()) {
    cfgpu_dns h = nullptr;
    SCK(cfgpu_ensemble_create(&r.grid, &r.flags, 1, s->precision, &h));
    s->used += cfgpu_rt::bytes(h);
    it = s->staging.emplace(r.key, h).first;
  }
  *out = it->second;
  return CFGPU_OK;
}

int finish(cfgpu_server_s* s, Request& r, cfgpu_dns h, int slot) {
  SCK(cfgpu_ensemble_get_field(h, slot, r.u.data(), r.q.data()));
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

// Start request r: its start-up steps in the staging DNS, then into a free slot of e.
int start_request(cfgpu_server_s* s, Request& r, Ens* e, int slot) {
  cfgpu_dns st = nullptr;
  SCK(make_staging(s, r, &st));
  SCK(cfgpu_ensemble_set_params(st, 0, &r.flags, nullptr, nullptr));
  SCK(cfgpu_rt::restart(st));
  SCK(cfgpu_ensemble_set_field(st, 0, r.u.data(), r.q.data()));
  r.t_start = now_s();
  r.status = ST_RUNNING;
  const int n0 = std::min(cfgpu_rt::startup_steps(st), r.nsteps);
  if (n0 > 0) {
    SCK(cfgpu_rt::advance_async(st, n0));
    if (cudaStreamSynchronize(cfgpu_rt::stream(st)) != cudaSuccess) return sfail(CFGPU_ECUDA, "staging step failed");
    r.done = n0;
  }
  if (r.done >= r.nsteps) return finish(s, r, st, 0);
  SCK(cfgpu_ensemble_set_params(e->h, slot, &r.flags, nullptr, nullptr));
  SCK(cfgpu_ensemble_load_slot(e->h, slot, st));
  e->slot_req[slot] = r.id;
  r.ens = -1;
  for (size_t i = 0; i < s->ens.size(); ++i)
    if (s->ens[i].get() == e) r.ens = (int)i;
  r.slot = slot;
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
      s->used -= e->bytes;
      cfgpu_dns_destroy(e->h);
      e.reset();
    }
}

int admit(cfgpu_server_s* s) {
  std::deque<long long> keep;
  bool dropped = false;
  while (!s->queue.empty()) {
    const long long id = s->queue.front();
    s->queue.pop_front();
    Request& r = *s->reqs[id];
    int slot = -1;
    Ens* e = find_slot(s, r.key, &slot);
    if (!e) {
      const long long est = cfgpu_rt::estimate_bytes(r.grid, r.flags, s->slots, s->precision) +
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
      int st = cfgpu_ensemble_create(&r.grid, &r.flags, s->slots, s->precision, &ne->h);
      if (st != CFGPU_OK) {
        r.status = ST_FAILED;
        r.err = cfgpu_last_error();
        continue;
      }
      ne->bytes = cfgpu_rt::bytes(ne->h);
      s->used += ne->bytes;
      ne->slot_req.assign(s->slots, -1);
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
  auto r = std::make_unique<Request>();
  r->id = s->next_id++;
  r->grid = *grid;
  r->flags = *flags;
  r->key = make_key(*grid, *flags);
  r->nsteps = nsteps;
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

cfgpu_status cfgpu_server_pump(cfgpu_server s, int max_steps, int* active) {
  if (!s || max_steps < 1) return sfail(CFGPU_EINVAL, "bad argument");
  SCK(admit(s));
  // advance: the largest step count that ends no running request early, capped by max_steps
  for (auto& e : s->ens) {
    if (!e) continue;
    int k = max_steps;
    for (long long id : e->slot_req)
      if (id >= 0) {
        const Request& r = *s->reqs[id];
        k = std::min(k, r.nsteps - r.done);
      }
    e->k = e->running() ? k : 0;
    if (e->k > 0) SCK(cfgpu_rt::advance_async(e->h, e->k));
  }
  for (auto& e : s->ens) {
    if (!e || e->k == 0) continue;
    if (cudaStreamSynchronize(cfgpu_rt::stream(e->h)) != cudaSuccess)
      return sfail(CFGPU_ECUDA, "ensemble step failed");
    s->steps_done += e->k;
    for (int i = 0; i < (int)e->slot_req.size(); ++i) {
      const long long id = e->slot_req[i];
      if (id < 0) continue;
      Request& r = *s->reqs[id];
      r.done += e->k;
      s->field_steps += e->k;
      if (r.done >= r.nsteps) {
        SCK(finish(s, r, e->h, i));
        e->slot_req[i] = -1;
      }
    }
    e->k = 0;
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
  return CFGPU_OK;
}

cfgpu_status cfgpu_server_destroy(cfgpu_server s) {
  if (!s) return CFGPU_OK;
  for (auto& e : s->ens)
    if (e) cfgpu_dns_destroy(e->h);
  for (auto& kv : s->staging) cfgpu_dns_destroy(kv.second);
  delete s;
  return CFGPU_OK;
}

}  // extern "C"
