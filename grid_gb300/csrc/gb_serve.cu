// gb_serve.cu -- a continuous-batching propagator-solve service on one GPU.
//
// Requests (Moebius DWF: geometry, Ls, mass, a seeded gauge field, nsrc Gaussian
// sources) enter a queue.  `slots` worker threads each own a CUDA stream; a worker admits
// a queued request as soon as its device-memory estimate fits what is left of the HBM
// budget (arrival order, or least work first, with an age bound after which the oldest
// request may not be passed), builds an FP64 and an inner-precision operator with nrhs = number of sources
// (so one multi-RHS Dslash launch reads each link once for all of the request's sources),
// generates the gauge field and the sources on the device, and runs the mixed-precision
// SchurRedBlackDiagMooeeSolve.  Requests that arrive while others run are admitted as
// slots and memory free up; their kernels overlap on the device through the streams.
// A request whose sources do not fit the budget together is solved in chunks of
// sources; one that does not fit with a single source is rejected at submission
// (GB_ERR_OOM).  The worker path allocates through the library's stream-ordered
// allocator, so no slot synchronises the device while the others run.  Each request's
// device work is bracketed by CUDA events on its slot's stream, which places it on the
// GPU's own timeline.
//
// Dry-run mode (flags bit 0) replaces the device work by a sleep of the request's
// dry_seconds, so the admission logic can be exercised without a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "gb_ops.h"

namespace gb {

// ---------------------------------------------------------------------------------------
// device generators: the same counter-based construction as gb_random.cpp
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t dmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double duniform(uint64_t seed, uint64_t ctr) {
  const uint64_t h = dmix64(dmix64(seed) ^ ctr);
  return double((h >> 11) + 1) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ double dnormal(uint64_t seed, uint64_t ctr) {
  const double u1 = duniform(seed, 2 * ctr), u2 = duniform(seed, 2 * ctr + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

struct DC {
  double re, im;
};
__device__ __forceinline__ DC cmul(DC a, DC b) { return DC{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

__device__ void m3mul(const DC (&a)[9], const DC (&b)[9], DC (&c)[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      DC s{0, 0};
      for (int k = 0; k < 3; k++) {
        const DC p = cmul(a[i * 3 + k], b[k * 3 + j]);
        s.re += p.re; s.im += p.im;
      }
      c[i * 3 + j] = s;
    }
}

__global__ void random_gauge_kernel(int64_t nlinks, double eps, uint64_t seed, double2* U) {
  const int64_t link = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (link >= nlinks) return;
  const uint64_t base = uint64_t(link) * 18;
  DC A[9], H[9], X[9];
  for (int i = 0; i < 9; i++) A[i] = DC{dnormal(seed, base + 2 * i), dnormal(seed, base + 2 * i + 1)};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      H[i * 3 + j] = DC{0.5 * (A[i * 3 + j].re + A[j * 3 + i].re), 0.5 * (A[i * 3 + j].im - A[j * 3 + i].im)};
  const double tr = (H[0].re + H[4].re + H[8].re) / 3.0;
  H[0].re -= tr; H[4].re -= tr; H[8].re -= tr;
  double nrm = 0;
  for (int i = 0; i < 9; i++) {
    X[i] = DC{-eps * H[i].im, eps * H[i].re};  // i eps H
    nrm += X[i].re * X[i].re + X[i].im * X[i].im;
  }
  nrm = sqrt(nrm);
  int k = 0;
  while (nrm > 0.5) { nrm *= 0.5; k++; }
  const double sc = ldexp(1.0, -k);
  DC Y[9], T[9], E[9], W[9];
  for (int i = 0; i < 9; i++) {
    Y[i] = DC{X[i].re * sc, X[i].im * sc};
    T[i] = DC{(i % 4 == 0) ? 1.0 : 0.0, 0.0};
    E[i] = T[i];
  }
  for (int n = 1; n <= 18; n++) {
    m3mul(T, Y, W);
    for (int i = 0; i < 9; i++) {
      T[i] = DC{W[i].re / n, W[i].im / n};
      E[i].re += T[i].re; E[i].im += T[i].im;
    }
  }
  for (int s = 0; s < k; s++) {
    m3mul(E, E, W);
    for (int i = 0; i < 9; i++) E[i] = W[i];
  }
  // reunitarise: rows 0, 1 orthonormal, row 2 = conj(row0 x row1)
  double n0 = 0;
  for (int j = 0; j < 3; j++) n0 += E[j].re * E[j].re + E[j].im * E[j].im;
  n0 = 1.0 / sqrt(n0);
  for (int j = 0; j < 3; j++) { E[j].re *= n0; E[j].im *= n0; }
  DC d{0, 0};
  for (int j = 0; j < 3; j++) {  // conj(row0) . row1
    d.re += E[j].re * E[3 + j].re + E[j].im * E[3 + j].im;
    d.im += E[j].re * E[3 + j].im - E[j].im * E[3 + j].re;
  }
  for (int j = 0; j < 3; j++) {
    const DC p = cmul(d, E[j]);
    E[3 + j].re -= p.re; E[3 + j].im -= p.im;
  }
  double n1 = 0;
  for (int j = 0; j < 3; j++) n1 += E[3 + j].re * E[3 + j].re + E[3 + j].im * E[3 + j].im;
  n1 = 1.0 / sqrt(n1);
  for (int j = 0; j < 3; j++) { E[3 + j].re *= n1; E[3 + j].im *= n1; }
  auto cross = [&](int a, int b) {  // conj(E0a E1b - E0b E1a)
    const DC p = cmul(E[a], E[3 + b]), q = cmul(E[b], E[3 + a]);
    return DC{p.re - q.re, -(p.im - q.im)};
  };
  E[6] = cross(1, 2);
  E[7] = cross(2, 0);
  E[8] = cross(0, 1);
  for (int i = 0; i < 9; i++) U[size_t(link) * 9 + i] = make_double2(E[i].re, E[i].im);
}

__global__ void random_gaussian_kernel(size_t n, uint64_t seed, double2* out) {
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_double2(dnormal(seed, uint64_t(2 * i)), dnormal(seed, uint64_t(2 * i + 1)));
}

}  // namespace gb

using namespace gb;

// ---------------------------------------------------------------------------------------
// server
// ---------------------------------------------------------------------------------------
struct gb_server_s {
  size_t budget = 0, used = 0, peak_used = 0;
  int slots = 1;
  unsigned flags = 0;
  int use_graphs = 0;
  int device = 0;
  double age_limit = 10.0;  // seconds the oldest request waits before nothing may pass it
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::deque<std::pair<int64_t, gb_request>> queue;
  std::vector<gb_request_result> done;
  std::vector<std::thread> workers;
  int running = 0, max_running = 0, max_queued = 0;
  int64_t next_id = 0, submitted = 0, finished = 0, cancelled = 0, rejected = 0;
  bool stop = false;
  struct Sample {
    double t;
    int queued, running;
  };
  std::vector<Sample> trace;
  cudaEvent_t origin = nullptr;  // the device timeline's zero, recorded at creation
  double origin_host = 0.0;      // host seconds since t0 when origin completed
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  void sample() {  // under mu
    max_queued = std::max(max_queued, int(queue.size()));
    trace.push_back(Sample{now(), int(queue.size()), running});
  }
};

namespace {

// device bytes a Moebius mixed-precision Schur solve of nsrc sources holds (operators,
// gauge staging, FP64 and inner-precision workspace); an upper estimate
size_t request_bytes(const gb_request& r, int nsrc) {
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= r.dims[k];
  const int64_t n5 = vol / 2 * r.Ls * (nsrc + ((r.Ls * nsrc) & 1));
  const size_t lo = r.inner_precision == GB_F16 ? 52 : 96;
  const size_t per_site4 = 1152 + 576 + 64 + 576;  // FP64 + FP32 links, neighbours, FP64 gauge staging
  return size_t(vol) * per_site4 + size_t(n5) * (26 * 192 + 12 * lo);
}

// work of one CG iteration (the shortest-first key): 4D volume x Ls x sources
double request_work(const gb_request& r) {
  double v = 1;
  for (int k = 0; k < 4; k++) v *= r.dims[k];
  return v * r.Ls * r.nsrc;
}
// largest chunk of a request's sources that fits the whole budget (0: none does)
int fitting_chunk(const gb_server_s* S, const gb_request& r) {
  int chunk = r.nsrc;
  while (chunk > 0 && request_bytes(r, chunk) > S->budget) chunk--;
  return chunk;
}
// The queue position to admit now, or -1 (under mu).  Default: the first in arrival order
// that fits what is left of the budget; FIFO (flags bit 2), or once the oldest has waited
// age_limit: only the oldest; shortest first (bit 3): the least work among those allowed.
int pick(gb_server_s* S, size_t* need, int* chunk) {
  const int n = int(S->queue.size());
  if (n == 0) return -1;
  const bool only_head = (S->flags & 4) || S->now() - S->queue.front().second.t_submit >= S->age_limit;
  int best = -1;
  double best_work = 0;
  for (int i = 0; i < (only_head ? 1 : n); i++) {
    const gb_request& r = S->queue[i].second;
    const int c = fitting_chunk(S, r);
    const size_t nb = request_bytes(r, c);
    if (S->used + nb > S->budget) continue;
    const double w = request_work(r);
    if (best < 0 || ((S->flags & 8) && w < best_work)) {
      best = i;
      best_work = w;
      *need = nb;
      *chunk = c;
      if (!(S->flags & 8)) break;
    }
  }
  return best;
}

int solve_request(gb_server_s* S, const gb_request& rq, int nsrc, uint64_t src_seed_offset, cudaStream_t st,
                  gb_request_result* out, double* sol_host, size_t sol_offset) {
  gb_op_t od = nullptr, of = nullptr;
  gb_field_t src = nullptr, sol = nullptr;
  double* dU = nullptr;
  double* dS = nullptr;
  int rc = GB_OK;
  const double ph[8] = {1, 0, 1, 0, 1, 0, -1, 0};
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= rq.dims[k];
  const size_t ncomplex = size_t(vol) * rq.Ls * 12 * nsrc;
  do {
    if ((rc = gb_mobius_create(rq.dims, rq.Ls, rq.mf, rq.M5, rq.b, rq.c, ph, GB_F64, nsrc, st, 0, &od))) break;
    if ((rc = gb_mobius_create(rq.dims, rq.Ls, rq.mf, rq.M5, rq.b, rq.c, ph, rq.inner_precision, nsrc, st, 0, &of))) break;
    if (cudaMallocAsync(reinterpret_cast<void**>(&dU), size_t(vol) * 36 * 16, st) != cudaSuccess) { rc = GB_ERR_OOM; break; }
    const int64_t nl = vol * 4;
    random_gauge_kernel<<<unsigned((nl + 127) / 128), 128, 0, st>>>(nl, rq.eps, rq.gauge_seed, reinterpret_cast<double2*>(dU));
    if ((rc = gb_op_import_gauge_device(od, dU))) break;
    if ((rc = gb_op_import_gauge_device(of, dU))) break;
    cudaFreeAsync(dU, st);
    dU = nullptr;
    if ((rc = gb_field_create(od, GB_FULL, GB_F64, &src))) break;
    if ((rc = gb_field_create(od, GB_FULL, GB_F64, &sol))) break;
    if (cudaMallocAsync(reinterpret_cast<void**>(&dS), ncomplex * 16, st) != cudaSuccess) { rc = GB_ERR_OOM; break; }
    random_gaussian_kernel<<<unsigned((ncomplex + 255) / 256), 256, 0, st>>>(
        ncomplex, rq.src_seed + src_seed_offset, reinterpret_cast<double2*>(dS));
    if ((rc = gb_field_import_device(src, dS))) break;
    gb_field_zero(sol);
    gb_cg_params P;
    gb_cg_params_default(&P);
    P.tolerance = rq.tolerance > 0 ? rq.tolerance : 1e-10;
    P.max_iterations = rq.max_iterations > 0 ? rq.max_iterations : 20000;
    P.use_graphs = S->use_graphs;
    gb_cg_result R;
    std::vector<double> unprec(nsrc);
    rc = gb_schur_solve(od, of, src, sol, &P, &R, unprec.data());
    out->iterations = std::max(out->iterations, R.iterations);
    out->reliable_updates += R.reliable_updates;
    out->cleanup_iterations = std::max(out->cleanup_iterations, R.cleanup_iterations);
    out->true_residual = std::max(out->true_residual, R.true_residual);
    for (double u : unprec) out->unprec_residual = std::max(out->unprec_residual, u);
    if (rc) break;
    std::vector<double> n2(nsrc);
    if ((rc = gb_field_norm2(sol, n2.data()))) break;
    for (int i = 0; i < nsrc; i++) out->solution_norm2 += n2[i];
    if (sol_host) {
      if ((rc = gb_field_export_device(sol, dS))) break;
      if (cudaMemcpyAsync(sol_host + sol_offset, dS, ncomplex * 16, cudaMemcpyDeviceToHost, st) != cudaSuccess) { rc = GB_ERR_CUDA; break; }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = GB_ERR_CUDA;
  } while (false);
  if (dU) cudaFreeAsync(dU, st);
  if (dS) cudaFreeAsync(dS, st);
  gb_field_destroy(src);
  gb_field_destroy(sol);
  gb_op_destroy(of);
  gb_op_destroy(od);
  return rc;
}

// device seconds of event e on the server's device timeline (-1 when unavailable)
double device_time(gb_server_s* S, cudaEvent_t e) {
  float ms = 0.f;
  if (!S->origin || cudaEventElapsedTime(&ms, S->origin, e) != cudaSuccess) return -1.0;
  return S->origin_host + ms * 1e-3;
}

void worker(gb_server_s* S) {
  const bool dry = S->flags & 1;
  if (!dry) cudaSetDevice(S->device);
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!dry) {
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
  }
  for (;;) {
    std::pair<int64_t, gb_request> item;
    size_t need = 0;
    int chunk = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      int at = -1;
      for (;;) {
        if (S->stop && S->queue.empty()) {
          lk.unlock();
          if (e0) cudaEventDestroy(e0);
          if (e1) cudaEventDestroy(e1);
          if (st) cudaStreamDestroy(st);
          return;
        }
        if ((at = pick(S, &need, &chunk)) >= 0) break;
        // wake at least when the oldest request reaches its age bound
        S->cv.wait_for(lk, std::chrono::milliseconds(50));
      }
      item = S->queue[at];
      S->queue.erase(S->queue.begin() + at);
      S->used += need;
      S->peak_used = std::max(S->peak_used, S->used);
      S->running++;
      S->max_running = std::max(S->max_running, S->running);
      S->sample();
    }
    const gb_request& rq = item.second;
    gb_request_result res;
    std::memset(&res, 0, sizeof(res));
    res.id = item.first;
    res.t_submit = rq.t_submit;
    res.t_start = S->now();
    res.nsrc = rq.nsrc;
    res.chunk = chunk;
    res.dev_start = res.dev_end = -1.0;
    if (dry) {
      std::this_thread::sleep_for(std::chrono::duration<double>(rq.dry_seconds));
      res.status = GB_OK;
    } else {
      cudaEventRecord(e0, st);
      int rc = GB_OK;
      for (int first = 0; first < rq.nsrc && rc == GB_OK; first += chunk) {
        const int n = std::min(chunk, rq.nsrc - first);
        int64_t vol = 1;
        for (int k = 0; k < 4; k++) vol *= rq.dims[k];
        rc = solve_request(S, rq, n, uint64_t(first) * 0x100000001ull, st, &res, rq.solution,
                           size_t(first) * size_t(vol) * rq.Ls * 24);
      }
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) == cudaSuccess) {
        res.dev_start = device_time(S, e0);
        res.dev_end = device_time(S, e1);
      }
      res.status = rc;
    }
    res.t_end = S->now();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->used -= need;
      S->running--;
      S->done.push_back(res);
      S->finished++;
      S->sample();
    }
    S->cv.notify_all();
    S->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

int gb_random_gauge_device(const int dims[4], double eps, uint64_t seed, double* U_dev, void* stream) {
  if (!dims || !U_dev) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= dims[k];
  const int64_t nl = vol * 4;
  random_gauge_kernel<<<unsigned((nl + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      nl, eps, seed, reinterpret_cast<double2*>(U_dev));
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int gb_random_gaussian_device(size_t n_complex, uint64_t seed, double* out_dev, void* stream) {
  if (!out_dev) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  random_gaussian_kernel<<<unsigned((n_complex + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n_complex, seed, reinterpret_cast<double2*>(out_dev));
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int gb_server_create(size_t hbm_budget_bytes, int slots, unsigned flags, gb_server_t* out) {
  if (!out || slots < 1 || hbm_budget_bytes == 0) { set_error("server: bad arguments"); return GB_ERR_BAD_ARG; }
  gb_server_s* S = new gb_server_s;
  S->budget = hbm_budget_bytes;
  S->slots = slots;
  S->flags = flags;
  S->use_graphs = (flags & 2) ? 2 : 0;  // the device-resident CG loop
  if (!(flags & 1)) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { delete S; set_error("no CUDA device"); return GB_ERR_NO_DEVICE; }
    cudaGetDevice(&S->device);
    // the device timeline's origin: an event that has completed at a known host time
    if (cudaEventCreate(&S->origin) == cudaSuccess) {
      cudaEventRecord(S->origin, nullptr);
      cudaEventSynchronize(S->origin);
      S->origin_host = S->now();
    } else {
      S->origin = nullptr;
    }
  }
  for (int i = 0; i < slots; i++) S->workers.emplace_back(worker, S);
  *out = S;
  return GB_OK;
}

int gb_request_bytes(const gb_request* r, size_t* bytes) {
  if (!r || !bytes || r->nsrc < 1) return GB_ERR_BAD_ARG;
  *bytes = request_bytes(*r, r->nsrc);
  return GB_OK;
}

int gb_server_submit(gb_server_t S, const gb_request* r, int64_t* id) {
  if (!S || !r || r->nsrc < 1 || r->Ls < 2 || (r->Ls & 1)) { set_error("server: bad request"); return GB_ERR_BAD_ARG; }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    gb_request q = *r;
    q.t_submit = S->now();
    const int64_t i = S->next_id++;
    S->submitted++;
    if (id) *id = i;
    if (fitting_chunk(S, q) == 0) {  // not even one source fits the whole budget
      gb_request_result res;
      std::memset(&res, 0, sizeof(res));
      res.id = i;
      res.status = GB_ERR_OOM;
      res.nsrc = q.nsrc;
      res.t_submit = res.t_start = res.t_end = q.t_submit;
      res.dev_start = res.dev_end = -1.0;
      S->done.push_back(res);
      S->finished++;
      S->rejected++;
    } else {
      S->queue.emplace_back(i, q);
    }
    S->sample();
  }
  S->cv.notify_all();
  S->cv_done.notify_all();
  return GB_OK;
}

int gb_server_set_age_limit(gb_server_t S, double seconds) {
  if (!S || !(seconds >= 0)) return GB_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  S->age_limit = seconds;
  return GB_OK;
}

int gb_server_cancel_queued(gb_server_t S, int64_t* n) {
  if (!S) return GB_ERR_BAD_ARG;
  int64_t k = 0;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    const double t = S->now();
    for (auto& it : S->queue) {
      gb_request_result res;
      std::memset(&res, 0, sizeof(res));
      res.id = it.first;
      res.status = GB_ERR_CANCELLED;
      res.nsrc = it.second.nsrc;
      res.t_submit = it.second.t_submit;
      res.t_start = res.t_end = t;
      res.dev_start = res.dev_end = -1.0;
      S->done.push_back(res);
      k++;
    }
    S->queue.clear();
    S->finished += k;
    S->cancelled += k;
    S->sample();
  }
  if (n) *n = k;
  S->cv.notify_all();
  S->cv_done.notify_all();
  return GB_OK;
}

int gb_server_trace(gb_server_t S, double* t, int* queued, int* running, int max, int* n) {
  if (!S || !n || max < 0) return GB_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  const int k = std::min<int>(max, int(S->trace.size()));
  for (int i = 0; i < k; i++) {
    if (t) t[i] = S->trace[i].t;
    if (queued) queued[i] = S->trace[i].queued;
    if (running) running[i] = S->trace[i].running;
  }
  *n = k;
  return GB_OK;
}

int gb_server_wait(gb_server_t S, int64_t count, double timeout_s) {
  if (!S) return GB_ERR_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  const bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                      [&] { return S->finished >= count; });
  return ok ? GB_OK : GB_ERR_TIMEOUT;
}

int gb_server_results(gb_server_t S, gb_request_result* out, int max, int* n) {
  if (!S || !n) return GB_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  const int k = std::min<int>(max, int(S->done.size()));
  for (int i = 0; i < k; i++) out[i] = S->done[i];
  S->done.erase(S->done.begin(), S->done.begin() + k);
  *n = k;
  return GB_OK;
}

int gb_server_stats(gb_server_t S, gb_server_stats_t* st) {
  if (!S || !st) return GB_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  st->budget_bytes = S->budget;
  st->used_bytes = S->used;
  st->peak_used_bytes = S->peak_used;
  st->running = S->running;
  st->max_running = S->max_running;
  st->queued = int(S->queue.size());
  st->submitted = S->submitted;
  st->finished = S->finished;
  st->now = S->now();
  st->cancelled = S->cancelled;
  st->rejected = S->rejected;
  st->max_queued = S->max_queued;
  return GB_OK;
}

int gb_server_destroy(gb_server_t S) {
  if (!S) return GB_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  for (auto& t : S->workers) t.join();
  if (S->origin) cudaEventDestroy(S->origin);
  delete S;
  return GB_OK;
}

}  // extern "C"
