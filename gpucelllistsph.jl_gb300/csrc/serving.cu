// serving.cu -- continuous-batching scheduler over the FP32 ensembles (host
// code; no counterpart in the reference, which solves one SPHProblem per
// call of stepsolve!/timesolve!, src/sphproblem.jl:204-345 and :420-511).
//
// Requests -- dam-break solves with a horizon in steps -- arrive over time.
// Each is admitted once it has arrived and the device has room for it (free
// HBM against the ensemble's bytes per particle, twice, for buffer growth,
// within a reserve) -- in arrival order, or, under the shortest-first policy,
// smallest work (particles x steps) first while its dimension's particles in
// flight stay within a cap -- joins the 2-D or 3-D ensemble, and advances
// together with every other admitted solve in chunks of at most `chunk`
// steps, cut at the nearest horizon so that each solve stops exactly at its
// own.  A finished solve's fields are read back and its slot is released,
// which admits the next.  An ensemble keeps its instances independent, so a
// solve's result does not depend on what else ran beside it.
//
// The scheduler reaches its ensembles, the free memory and the clock
// through a backend table: the library's own (ens_*, cudaMemGetInfo, a
// steady clock), or a caller's (host-side tests drive the same scheduling
// against a fake ensemble).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <thread>
#include <vector>
#include "gcsph_common.cuh"

using namespace gcsph;

namespace {

enum { RQ_QUEUED = 0, RQ_RUNNING = 1, RQ_DONE = 2 };

struct SrvReq {
  int32_t D = 2;
  int64_t n = 0;
  int64_t steps = 0, remaining = 0;
  double arrival = 0, admitted = -1, done = -1;
  int32_t slot = -1;
  int state = RQ_QUEUED;
  // inputs until admission (library backend)
  std::vector<double> x, v, rho;
  std::vector<int32_t> ptype;
  gcsph_ens_params prm{};
  bool has_v = false;
  // results at the horizon, per field (library backend)
  std::vector<double> res[6];
};

}  // namespace

struct gcsph_srv {
  gcsph_srv_backend be{};
  bool own = false;        // the library's backend
  void* stream = nullptr;
  // the library's backend, no stream given: streams per dimension, so the
  // 2-D and 3-D ensembles' chunks run side by side -- [d][0] at the lowest
  // priority, [d][1] at the highest (shortest first: the dimension holding
  // the solve with the least work left runs on its high-priority stream)
  cudaStream_t dim_st[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // wall seconds per step of each dimension's last chunk (library backend):
  // the faster dimension takes more steps per round, so that a round's two
  // chunks take about the same time and neither dimension waits on the other
  double spp[2] = {0.0, 0.0};
  int32_t chunk = 64;
  double reserve = 0.1;
  int32_t policy = GCSPH_SRV_ARRIVAL;
  int64_t cap[2] = {0, 0};  // shortest-first: particles in flight per dimension (0: no cap)
  double max_wait = 0;      // shortest-first: a solve waiting this long ignores the cap (0: never)
  uint32_t fields = 7;     // bit f: read back GCSPH_ENS field f at the horizon
  gcsph_ens* ens[2] = {nullptr, nullptr};
  std::vector<SrvReq> req;
  std::chrono::steady_clock::time_point t0;
  int64_t particle_steps = 0;
  double last_done = 0;
};

namespace {

// ---- the library's backend ------------------------------------------------
gcsph_ens*& ens_of(gcsph_srv* s, int32_t D) { return s->ens[D == 3 ? 1 : 0]; }

int own_add(void* ctx, int32_t D, int32_t rid, int32_t* slot) {
  gcsph_srv* s = (gcsph_srv*)ctx;
  gcsph_ens*& e = ens_of(s, D);
  int rc;
  void* st = s->dim_st[D == 3 ? 1 : 0][0] ? (void*)s->dim_st[D == 3 ? 1 : 0][0] : s->stream;
  if (!e && (rc = ens_create(D, st, &e))) return rc;
  SrvReq& r = s->req[rid];
  rc = ens_add(e, r.n, r.x.data(), r.has_v ? r.v.data() : nullptr, r.rho.data(), r.ptype.data(), &r.prm, slot);
  if (rc) return rc;
  // the inputs live on the device now
  std::vector<double>().swap(r.x);
  std::vector<double>().swap(r.v);
  std::vector<double>().swap(r.rho);
  std::vector<int32_t>().swap(r.ptype);
  return GCSPH_OK;
}

int own_remove(void* ctx, int32_t D, int32_t slot) { return ens_remove(ens_of((gcsph_srv*)ctx, D), slot); }

int own_step(void* ctx, int32_t D, int32_t n) { return ens_step(ens_of((gcsph_srv*)ctx, D), n); }

int own_harvest(void* ctx, int32_t D, int32_t slot, int32_t rid) {
  gcsph_srv* s = (gcsph_srv*)ctx;
  SrvReq& r = s->req[rid];
  for (int f = 0; f < 6; ++f) {
    if (!(s->fields & (1u << f))) continue;
    const int comps = (f == GCSPH_ENS_X || f == GCSPH_ENS_V) ? D : 1;
    r.res[f].resize((size_t)comps * (size_t)r.n);
    int rc = ens_get(ens_of(s, D), slot, f, r.res[f].data());
    if (rc) return rc;
  }
  return GCSPH_OK;
}

int64_t own_free_bytes(void*) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (int64_t)fr;
}

int64_t own_bpp(void*, int32_t D) {
  int64_t b = 0;
  return ens_bytes_per_particle(D, &b) == GCSPH_OK ? b : INT64_MAX / 4;
}

double now_of(gcsph_srv* s) {
  if (s->be.now) return s->be.now(s->be.ctx);
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

bool fits(gcsph_srv* s, const SrvReq& r) {
  const double need = (double)r.n * (double)s->be.bytes_per_particle(s->be.ctx, r.D) * 2.0;
  return need <= (1.0 - s->reserve) * (double)s->be.free_bytes(s->be.ctx);
}

bool any_running(const gcsph_srv* s) {
  for (const SrvReq& r : s->req)
    if (r.state == RQ_RUNNING) return true;
  return false;
}

// numpy's default percentile: linear between the closest ranks
double percentile(std::vector<double> v, double p) {
  if (v.empty()) return NAN;
  std::sort(v.begin(), v.end());
  const double pos = (double)(v.size() - 1) * p / 100.0;
  const size_t lo = (size_t)std::floor(pos), hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
}

// one round: admit what has arrived and fits (arrival order, or smallest
// work first within the caps), then one chunk of every ensemble with running
// solves, then release the finished ones
int round(gcsph_srv* s, int* advanced) {
  *advanced = 0;
  const double now = now_of(s);
  std::vector<size_t> order;
  for (size_t i = 0; i < s->req.size(); ++i)
    if (s->req[i].state == RQ_QUEUED && s->req[i].arrival <= now) order.push_back(i);
  const bool shortest = s->policy == GCSPH_SRV_SHORTEST;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    const SrvReq &ra = s->req[a], &rb = s->req[b];
    if (shortest) {
      const double wa = (double)ra.n * (double)ra.steps, wb = (double)rb.n * (double)rb.steps;
      if (wa != wb) return wa < wb;
    }
    return ra.arrival < rb.arrival;
  });
  int64_t inflight[2] = {0, 0};
  for (const SrvReq& r : s->req)
    if (r.state == RQ_RUNNING) inflight[r.D == 3 ? 1 : 0] += r.n;
  for (size_t i : order) {
    SrvReq& r = s->req[i];
    const int di = r.D == 3 ? 1 : 0;
    // within the cap, except that an idle dimension takes any solve and a
    // solve that has waited max_wait is not held back by it
    const bool aged = s->max_wait > 0 && now - r.arrival >= s->max_wait;
    if (shortest && !aged && s->cap[di] > 0 && inflight[di] > 0 && inflight[di] + r.n > s->cap[di]) continue;
    if (!fits(s, r)) continue;
    int32_t slot = -1;
    int rc = s->be.add(s->be.ctx, r.D, (int32_t)i, &slot);
    if (rc) return rc;
    r.slot = slot;
    r.state = RQ_RUNNING;
    r.admitted = now_of(s);
    r.remaining = r.steps;
    inflight[di] += r.n;
  }
  int64_t kd[2] = {s->chunk, s->chunk}, lived[2] = {0, 0}, left[2] = {INT64_MAX, INT64_MAX};
  double least[2] = {INFINITY, INFINITY};  // least work (particles x steps) left of a running solve
  for (const SrvReq& r : s->req)
    if (r.state == RQ_RUNNING) {
      const int di = r.D == 3 ? 1 : 0;
      left[di] = std::min(left[di], r.remaining);
      lived[di] += r.n;
      least[di] = std::min(least[di], (double)r.n * (double)r.remaining);
    }
  const bool both = s->dim_st[0][0] && s->dim_st[1][0] && lived[0] > 0 && lived[1] > 0;
  if (both && s->spp[0] > 0 && s->spp[1] > 0) {
    // the dimension that is faster per step takes a power-of-two multiple of
    // the chunk (at most 16), so that both chunks take about the same time
    const int slow = s->spp[0] >= s->spp[1] ? 0 : 1, fast = 1 - slow;
    const double ratio = s->spp[slow] / s->spp[fast];
    int64_t k = s->chunk;
    while (k < 16 * (int64_t)s->chunk && (double)(2 * k) <= (double)s->chunk * ratio) k *= 2;
    kd[fast] = k;
  }
  for (int di = 0; di < 2; ++di) kd[di] = std::min(kd[di], left[di]);
  if (both) {
    // shortest first: the solve with the least work left gets the GPU first
    const int hi = s->policy == GCSPH_SRV_SHORTEST ? (least[0] <= least[1] ? 0 : 1) : -1;
    for (int di = 0; di < 2; ++di) {
      int rc = ens_set_stream(s->ens[di], s->dim_st[di][di == hi ? 1 : 0]);
      if (rc) return rc;
    }
  }
  auto timed_step = [&](int di) {
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = s->be.step(s->be.ctx, 2 + di, (int32_t)kd[di]);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc == GCSPH_OK && kd[di] > 0) s->spp[di] = sec / (double)kd[di];
    return rc;
  };
  int rcd[2] = {GCSPH_OK, GCSPH_OK};
  if (both) {
    // both ensembles run: the 3-D chunk from a second host thread, on its own
    // stream, while this thread runs the 2-D one (an error's message is
    // carried back: the library keeps it per thread)
    std::string msg3;
    std::thread t([&] {
      rcd[1] = timed_step(1);
      if (rcd[1]) msg3 = gcsph_last_error();
    });
    rcd[0] = timed_step(0);
    t.join();
    if (rcd[0]) return rcd[0];
    if (rcd[1]) return fail(rcd[1], "%s", msg3.c_str());
  } else {
    for (int di = 0; di < 2; ++di)
      if (lived[di] > 0 && (rcd[di] = timed_step(di))) return rcd[di];
  }
  for (int32_t D = 2; D <= 3; ++D) {
    const int di = D == 3 ? 1 : 0;
    const int64_t k = kd[di], live = lived[di];
    if (live == 0) continue;
    int rc;
    *advanced = 1;
    s->particle_steps += k * live;
    for (size_t i = 0; i < s->req.size(); ++i) {
      SrvReq& r = s->req[i];
      if (r.state != RQ_RUNNING || r.D != D) continue;
      r.remaining -= k;
      if (r.remaining > 0) continue;
      if ((rc = s->be.harvest(s->be.ctx, D, r.slot, (int32_t)i))) return rc;
      if ((rc = s->be.remove(s->be.ctx, D, r.slot))) return rc;
      r.state = RQ_DONE;
      r.done = now_of(s);
      s->last_done = r.done;
    }
  }
  return GCSPH_OK;
}

}  // namespace

extern "C" {

int srv_create(void* stream, int32_t chunk, double reserve, uint32_t fields, const gcsph_srv_backend* backend,
               gcsph_srv** out) {
  if (!out) return fail(GCSPH_EINVAL, "null argument");
  *out = nullptr;
  if (chunk < 1) return fail(GCSPH_EINVAL, "chunk %d (at least 1)", (int)chunk);
  if (!(reserve >= 0.0 && reserve < 1.0)) return fail(GCSPH_EINVAL, "reserve %g (0 .. 1)", reserve);
  if (fields >= (1u << 6)) return fail(GCSPH_EINVAL, "fields mask 0x%x (bits 0..5)", fields);
  if (backend && (!backend->add || !backend->remove || !backend->step || !backend->harvest ||
                  !backend->free_bytes || !backend->bytes_per_particle))
    return fail(GCSPH_EINVAL, "incomplete serving backend");
  gcsph_srv* s = new gcsph_srv();
  s->stream = stream;
  s->chunk = chunk;
  s->reserve = reserve;
  s->fields = fields;
  s->t0 = std::chrono::steady_clock::now();
  if (backend) {
    s->be = *backend;
  } else {
    s->own = true;
    int lo = 0, hi = 0;
    if (!stream && cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess) {
      for (auto& pair : s->dim_st)
        for (int k = 0; k < 2; ++k)
          if (cudaStreamCreateWithPriority(&pair[k], cudaStreamNonBlocking, k ? hi : lo) != cudaSuccess) {
            cudaGetLastError();
            pair[k] = nullptr;
          }
      for (auto& pair : s->dim_st)
        if (!pair[0] || !pair[1]) {
          for (auto& q : s->dim_st)
            for (cudaStream_t& st : q) {
              if (st) cudaStreamDestroy(st);
              st = nullptr;
            }
          break;
        }
    }
    cudaGetLastError();
    s->be.ctx = s;
    s->be.add = own_add;
    s->be.remove = own_remove;
    s->be.step = own_step;
    s->be.harvest = own_harvest;
    s->be.free_bytes = own_free_bytes;
    s->be.bytes_per_particle = own_bpp;
    s->be.now = nullptr;
  }
  *out = s;
  return GCSPH_OK;
}

void srv_destroy(gcsph_srv* s) {
  if (!s) return;
  for (gcsph_ens* e : s->ens)
    if (e) ens_destroy(e);
  for (auto& pair : s->dim_st)
    for (cudaStream_t st : pair)
      if (st) cudaStreamDestroy(st);
  delete s;
}

int srv_submit(gcsph_srv* s, int32_t D, int64_t n, const double* x, const double* v, const double* rho,
               const int32_t* ptype, const gcsph_ens_params* p, int64_t steps, double arrival, int32_t* rid) {
  if (!s || !rid) return fail(GCSPH_EINVAL, "null argument");
  if (D != 2 && D != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", (int)D);
  if (n <= 0 || steps < 1) return fail(GCSPH_EINVAL, "n = %lld, steps = %lld", (long long)n, (long long)steps);
  SrvReq r;
  r.D = D;
  r.n = n;
  r.steps = r.remaining = steps;
  r.arrival = arrival >= 0 ? arrival : now_of(s);
  if (s->own) {
    if (!x || !rho || !ptype || !p) return fail(GCSPH_EINVAL, "null input array");
    r.x.assign(x, x + (size_t)D * (size_t)n);
    if (v) {
      r.v.assign(v, v + (size_t)D * (size_t)n);
      r.has_v = true;
    }
    r.rho.assign(rho, rho + n);
    r.ptype.assign(ptype, ptype + n);
    r.prm = *p;
  }
  s->req.push_back(std::move(r));
  *rid = (int32_t)(s->req.size() - 1);
  return GCSPH_OK;
}

int srv_set_policy(gcsph_srv* s, int32_t policy, int64_t cap2d, int64_t cap3d, double max_wait) {
  if (!s) return fail(GCSPH_EINVAL, "null handle");
  if (policy != GCSPH_SRV_ARRIVAL && policy != GCSPH_SRV_SHORTEST)
    return fail(GCSPH_EINVAL, "policy %d (GCSPH_SRV_ARRIVAL or GCSPH_SRV_SHORTEST)", (int)policy);
  if (cap2d < 0 || cap3d < 0) return fail(GCSPH_EINVAL, "negative particle cap");
  if (!(max_wait >= 0)) return fail(GCSPH_EINVAL, "max_wait %g (0: never)", max_wait);
  s->policy = policy;
  s->cap[0] = cap2d;
  s->cap[1] = cap3d;
  s->max_wait = max_wait;
  return GCSPH_OK;
}

int srv_get_policy(gcsph_srv* s, int32_t* policy, int64_t* cap2d, int64_t* cap3d, double* max_wait) {
  if (!s) return fail(GCSPH_EINVAL, "null handle");
  if (policy) *policy = s->policy;
  if (cap2d) *cap2d = s->cap[0];
  if (cap3d) *cap3d = s->cap[1];
  if (max_wait) *max_wait = s->max_wait;
  return GCSPH_OK;
}

int srv_progress(gcsph_srv* s, int32_t* running, int32_t* queued) {
  if (!s) return fail(GCSPH_EINVAL, "null handle");
  int adv = 0;
  int rc = round(s, &adv);
  if (rc) return rc;
  int32_t nr = 0, nq = 0;
  for (const SrvReq& r : s->req) {
    nr += r.state == RQ_RUNNING;
    nq += r.state == RQ_QUEUED;
  }
  if (running) *running = nr;
  if (queued) *queued = nq;
  return GCSPH_OK;
}

int srv_run(gcsph_srv* s) {
  if (!s) return fail(GCSPH_EINVAL, "null handle");
  for (;;) {
    int adv = 0;
    int rc = round(s, &adv);
    if (rc) return rc;
    double next = INFINITY;
    bool queued = false, arrived = false;
    const double now = now_of(s);
    for (const SrvReq& r : s->req)
      if (r.state == RQ_QUEUED) {
        queued = true;
        if (r.arrival <= now) arrived = true;
        next = std::min(next, r.arrival);
      }
    if (!queued && !any_running(s)) return GCSPH_OK;
    if (adv || any_running(s)) continue;
    if (arrived) {
      // nothing runs and an arrived solve still has no room: it never will
      for (const SrvReq& r : s->req)
        if (r.state == RQ_QUEUED && r.arrival <= now)
          return fail(GCSPH_ECAPACITY, "a request of %lld particles does not fit in the device's free memory",
                      (long long)r.n);
    }
    const double wait = next - now;
    if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
  }
}

int srv_request(gcsph_srv* s, int32_t rid, int32_t* state, double* arrival, double* admitted, double* done) {
  if (!s) return fail(GCSPH_EINVAL, "null handle");
  if (rid < 0 || (size_t)rid >= s->req.size()) return fail(GCSPH_EINVAL, "no request %d", (int)rid);
  const SrvReq& r = s->req[rid];
  if (state) *state = r.state;
  if (arrival) *arrival = r.arrival;
  if (admitted) *admitted = r.admitted;
  if (done) *done = r.done;
  return GCSPH_OK;
}

int srv_result(gcsph_srv* s, int32_t rid, int32_t field, double* out_host) {
  if (!s || !out_host) return fail(GCSPH_EINVAL, "null argument");
  if (rid < 0 || (size_t)rid >= s->req.size()) return fail(GCSPH_EINVAL, "no request %d", (int)rid);
  if (!s->own) return fail(GCSPH_ESTATE, "results stay with the caller's backend");
  const SrvReq& r = s->req[rid];
  if (r.state != RQ_DONE) return fail(GCSPH_ESTATE, "request %d has not reached its horizon", (int)rid);
  if (field < 0 || field >= 6 || !(s->fields & (1u << field)))
    return fail(GCSPH_EINVAL, "field %d was not read back (fields mask 0x%x)", (int)field, s->fields);
  std::copy(r.res[field].begin(), r.res[field].end(), out_host);
  return GCSPH_OK;
}

int srv_stats(gcsph_srv* s, gcsph_srv_stats* st) {
  if (!s || !st) return fail(GCSPH_EINVAL, "null argument");
  std::vector<double> lat;
  for (const SrvReq& r : s->req)
    if (r.state == RQ_DONE) lat.push_back(r.done - r.arrival);
  double mean = NAN;
  if (!lat.empty()) {
    mean = 0;
    for (double l : lat) mean += l;
    mean /= (double)lat.size();
  }
  st->requests = (int32_t)s->req.size();
  st->completed = (int32_t)lat.size();
  st->particle_steps = s->particle_steps;
  st->wall_s = s->last_done;
  st->p50_s = percentile(lat, 50.0);
  st->p99_s = percentile(lat, 99.0);
  st->mean_s = mean;
  return GCSPH_OK;
}

}  // extern "C"
