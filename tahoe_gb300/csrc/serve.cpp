// Served RVE stream inside the library (configuration 5): a request loop in
// C++ behind the C ABI (tg_serve_*).
//
// A caller submits RVE requests (side n, macroscopic F) as they arrive and
// polls for the volume-averaged first Piola stress.  A pool of lanes serves
// them; each lane is a host thread owning a context (its own CUDA stream and
// resident RVE templates: one mesh structure per side length, registered
// once with tg_template_add).  A free lane takes the requests that have
// arrived, in arrival order, while
//   * the batch stays within max_batch requests,
//   * the bytes of every batch in flight stay within the device-memory
//     budget (per-RVE estimate), and
//   * the batch's predicted solve time stays within the latency target (a
//     model ms = a + b * elements fitted to the lane pool's own batches);
// composes the batch mesh on the device (tg_mesh_compose), runs the affine
// predictor and the segmented Newton (one Krylov solve per RVE, an RVE that
// fails fails alone) and reports every request's stress and status.  Lanes
// run concurrently, so batches from several lanes overlap on the GPU and a
// request that arrives while others are being solved is admitted by the
// next free lane.  Requests of a batch that failed (the batch as a whole:
// a CUDA, memory or bad-Jacobian error) are retried alone.
//
// The RVE is the benchmark's: an n x n x n hex8 unit cube (nodes x-fastest,
// coordinates i/n), a centred spherical inclusion of radius 0.3 (elements by
// centroid) with ten times the matrix moduli (Simo neo-Hookean, matrix mu 1,
// kappa 10), every boundary node prescribed to the affine displacement
// (F - I) X.  No reference counterpart: the reference has no FE^2 driver.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tg_internal.h"

namespace {

double now_ms(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Mesh arrays of the RVE of side n, as tg_template_add takes them.
struct RveMesh {
  int n = 0, nnd = 0, nel = 0;
  std::vector<double> coords;  // SoA
  std::vector<int> conn, eqnos, blocks;
};

RveMesh make_rve(int n) {
  RveMesh m;
  m.n = n;
  const int np = n + 1;
  m.nnd = np * np * np;
  m.nel = n * n * n;
  std::vector<double> xs(np);
  const double step = 1.0 / n;
  for (int i = 0; i < np; ++i) xs[i] = i == n ? 1.0 : i * step;  // numpy linspace(0, 1, n + 1)
  m.coords.resize(3 * (size_t)m.nnd);
  std::vector<char> bnd(m.nnd, 0);
  for (int k = 0; k < np; ++k)
    for (int j = 0; j < np; ++j)
      for (int i = 0; i < np; ++i) {
        const int a = i + np * (j + np * k);
        m.coords[a] = xs[i];
        m.coords[m.nnd + a] = xs[j];
        m.coords[2 * (size_t)m.nnd + a] = xs[k];
        bnd[a] = (i == 0 || i == n || j == 0 || j == n || k == 0 || k == n) ? 1 : 0;
      }
  m.conn.resize(8 * (size_t)m.nel);
  m.blocks.resize(m.nel);
  auto nid = [&](int i, int j, int k) { return i + np * (j + np * k); };
  int e = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i, ++e) {
        const int v[8] = {nid(i, j, k),         nid(i + 1, j, k),     nid(i + 1, j + 1, k),     nid(i, j + 1, k),
                          nid(i, j, k + 1),     nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
        double c[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 8; ++a) {
          m.conn[8 * (size_t)e + a] = v[a];
          for (int d = 0; d < 3; ++d) c[d] += m.coords[(size_t)d * m.nnd + v[a]];
        }
        double r2 = 0.0;
        for (int d = 0; d < 3; ++d) {
          const double x = c[d] / 8.0 - 0.5;
          r2 += x * x;
        }
        m.blocks[e] = std::sqrt(r2) < 0.3 ? 1 : 0;
      }
  // NodeManagerT::SetEquationNumbers: boundary dofs prescribed
  m.eqnos.assign(3 * (size_t)m.nnd, 0);
  int q = 0;
  for (int a = 0; a < m.nnd; ++a)
    for (int d = 0; d < 3; ++d) m.eqnos[3 * (size_t)a + d] = bnd[a] ? -1 : ++q;
  return m;
}

// device bytes one RVE of side n holds while solved (estimate)
double rve_bytes(int n, int precision) {
  const double s = precision == TG_MIXED ? 4.0 : 8.0;
  const double nel = (double)n * n * n, nnd = (double)(n + 1) * (n + 1) * (n + 1);
  return nel * (432 * s + 256 + 8 * 32 + 128 + 8 * 25 * 8) + nnd * (27 * (9 * s + 8) + 10 * 16 + 6 * 4 * s + 64);
}

}  // namespace

struct tg_server {
  struct Req {
    int n = 0;
    double F[9];
    double t_arrive = 0.0, t_start = -1.0, t_finish = -1.0;
    int status = 0;
    bool done = false;
    double P[9];
  };
  int device = 0, lanes = 1, max_batch = 1, precision = TG_MIXED, precond = TG_PRECOND_BLOCK_JACOBI;
  double rel_tol = 1e-8, lin_rel_tol = 1e-4, budget = 0.0, target_ms = 0.0;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<long long> ready;
  std::deque<Req> reqs;  // by id (stable addresses)
  double inflight = 0.0;
  bool stop = false;
  int busy = 0, max_busy = 0;
  long long batches = 0, batched_requests = 0, retried = 0, completed = 0;
  // batch-time model ms = a + b * elements (least squares over the batches
  // seen, older batches weighted down)
  double sw = 0.0, sx = 0.0, sy = 0.0, sxx = 0.0, sxy = 0.0;
  std::string err;
  std::vector<std::thread> threads;

  double predict_ms(double elements) {
    const double det = sw * sxx - sx * sx;
    if (sw < 2.0 || det <= 1e-12 * sw * sxx) return 0.0;  // no model yet: admission by size and memory
    const double b = (sw * sxy - sx * sy) / det, a = (sy - b * sx) / sw;
    return std::max(0.0, a) + std::max(0.0, b) * elements;
  }
  void observe(double elements, double ms) {
    const double f = 0.98;
    sw = f * sw + 1.0;
    sx = f * sx + elements;
    sy = f * sy + ms;
    sxx = f * sxx + elements * elements;
    sxy = f * sxy + elements * ms;
  }
};

namespace {

struct Lane {
  tg_context* ctx = nullptr;
  std::map<int, int> tpl;  // side n -> template id
};

int lane_setup(tg_server* S, Lane& L) {
  int s = tg_create(&L.ctx, S->device);
  if (s) return s;
  s = tg_element_set(L.ctx, TG_TOTAL_LAGRANGIAN);
  const double matrix[2] = {1.0, 10.0}, inclusion[2] = {10.0, 100.0};
  if (!s) s = tg_material_set(L.ctx, 0, TG_MAT_FS_SIMO, matrix, 2);
  if (!s) s = tg_material_set(L.ctx, 1, TG_MAT_FS_SIMO, inclusion, 2);
  return s;
}

int template_of(Lane& L, int n, int* id) {
  auto it = L.tpl.find(n);
  if (it != L.tpl.end()) {
    *id = it->second;
    return TG_OK;
  }
  const RveMesh m = make_rve(n);
  int tid = -1;
  const int s = tg_template_add(L.ctx, m.nnd, m.coords.data(), m.nel, m.conn.data(), m.eqnos.data(),
                                m.blocks.data(), &tid);
  if (s) return s;
  L.tpl[n] = tid;
  *id = tid;
  return TG_OK;
}

// Solves the batch on the lane's context; st/P per request.  Returns a
// batch-level error (CUDA, memory, bad Jacobian, ...) or TG_OK with the
// per-RVE statuses.
int solve_batch(tg_server* S, Lane& L, const std::vector<int>& ns, const std::vector<const double*>& Fs,
                std::vector<int>& st, std::vector<double>& P) {
  const int k = (int)ns.size();
  std::vector<int> ids(k);
  for (int i = 0; i < k; ++i) {
    const int s = template_of(L, ns[i], &ids[i]);
    if (s) return s;
  }
  int s = tg_mesh_compose(L.ctx, k, ids.data());
  if (s) return s;
  std::vector<double> F(9 * (size_t)k);
  for (int i = 0; i < k; ++i) std::memcpy(&F[9 * (size_t)i], Fs[i], 9 * sizeof(double));
  tg_newton_params prm{};
  prm.rel_tol = S->rel_tol;
  prm.abs_tol = 0.0;
  prm.div_tol = 1e3;
  prm.max_iterations = 20;
  prm.precision = S->precision;
  prm.precond = S->precond;
  prm.lin_rel_tol = S->lin_rel_tol;
  prm.lin_max_it = 20000;
  int its = 0;
  s = tg_predict_affine(L.ctx, F.data(), &prm, &its);
  if (s) return s;
  tg_newton_report rep;
  std::vector<double> rel(k);
  st.assign(k, 0);
  s = tg_newton_solve_segmented(L.ctx, &prm, &rep, rel.data(), st.data());
  // RVE failures are reported per RVE; anything else ends the batch
  if (s && s != TG_ERR_NOT_CONVERGED && s != TG_ERR_DIVERGED && s != TG_ERR_NAN) return s;
  P.assign(9 * (size_t)k, 0.0);
  std::vector<double> vol(k, 1.0);
  return tg_segment_average_stress(L.ctx, vol.data(), P.data());
}

void lane_loop(tg_server* S, int lid) {
  Lane L;
  int setup = lane_setup(S, L);
  if (setup) {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->err.empty()) S->err = "lane " + std::to_string(lid) + ": context set-up failed";
  }
  for (;;) {
    std::vector<long long> take;
    std::vector<int> ns;
    std::vector<double> Fv;  // 9 per request, copied under the lock (the request list grows meanwhile)
    double used = 0.0, elements = 0.0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || !S->ready.empty(); });
      if (S->ready.empty()) break;  // stop requested and nothing left
      const double room = S->budget - S->inflight;
      while (!S->ready.empty() && (int)take.size() < S->max_batch) {
        const long long id = S->ready.front();
        const int n = S->reqs[id].n;
        const double b = rve_bytes(n, S->precision), el = (double)n * n * n;
        if (!take.empty()) {
          if (used + b > room) break;
          if (S->target_ms > 0.0 && S->predict_ms(elements + el) > S->target_ms) break;
        } else if (used + b > room && S->inflight > 0.0) {
          break;  // wait for memory to free up
        }
        take.push_back(id);
        used += b;
        elements += el;
        S->ready.pop_front();
      }
      if (take.empty()) {
        // memory is held by other lanes: wait for a batch to finish
        S->cv_done.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      S->inflight += used;
      S->busy += 1;
      S->max_busy = std::max(S->max_busy, S->busy);
      const double ts = now_ms(S->t0);
      for (long long id : take) {
        tg_server::Req& q = S->reqs[id];
        q.t_start = ts;
        ns.push_back(q.n);
        Fv.insert(Fv.end(), q.F, q.F + 9);
      }
    }
    const int k = (int)take.size();
    std::vector<const double*> Fs(k);
    for (int i = 0; i < k; ++i) Fs[i] = &Fv[9 * (size_t)i];
    const double tb = now_ms(S->t0);
    std::vector<int> st;
    std::vector<double> P;
    int s = setup ? setup : solve_batch(S, L, ns, Fs, st, P);
    const double batch_ms = now_ms(S->t0) - tb;
    if (s) {
      st.assign(k, s);
      P.assign(9 * (size_t)k, 0.0);
    }
    int retried = 0;
    if (k > 1 && !setup)
      for (int i = 0; i < k; ++i) {
        if (st[i] == 0) continue;
        // a failed request is retried alone
        std::vector<int> st1;
        std::vector<double> P1;
        const int s1 = solve_batch(S, L, {ns[i]}, {Fs[i]}, st1, P1);
        st[i] = s1 ? s1 : st1[0];
        if (!s1) std::memcpy(&P[9 * (size_t)i], P1.data(), 9 * sizeof(double));
        ++retried;
      }
    {
      std::lock_guard<std::mutex> g(S->mu);
      const double te = now_ms(S->t0);
      for (int i = 0; i < k; ++i) {
        tg_server::Req& q = S->reqs[take[i]];
        q.status = st[i];
        std::memcpy(q.P, &P[9 * (size_t)i], 9 * sizeof(double));
        q.t_finish = te;
        q.done = true;
      }
      if (!s) S->observe(elements, batch_ms);
      S->inflight -= used;
      S->busy -= 1;
      S->batches += 1;
      S->batched_requests += k;
      S->retried += retried;
      S->completed += k;
      if (s && S->err.empty()) S->err = tg_last_error(L.ctx);
    }
    S->cv_done.notify_all();
  }
  if (L.ctx) tg_destroy(L.ctx);
}

}  // namespace

extern "C" {

int tg_serve_create(tg_server** out, int device, int lanes, int max_batch, double budget_bytes, int precision,
                    int precond, double rel_tol, double lin_rel_tol, double target_batch_ms) {
  if (!out || lanes < 1 || lanes > 64 || max_batch < 1 || max_batch > 65535 || budget_bytes <= 0.0 ||
      (precision != TG_FP64 && precision != TG_MIXED) ||
      (precond != TG_PRECOND_JACOBI && precond != TG_PRECOND_BLOCK_JACOBI) || !(rel_tol > 0.0) ||
      !(lin_rel_tol > 0.0) || target_batch_ms < 0.0)
    return TG_ERR_ARG;
  tg_server* S = new tg_server();
  S->device = device;
  S->lanes = lanes;
  S->max_batch = max_batch;
  S->budget = budget_bytes;
  S->precision = precision;
  S->precond = precond;
  S->rel_tol = rel_tol;
  S->lin_rel_tol = lin_rel_tol;
  S->target_ms = target_batch_ms;
  S->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < lanes; ++i) S->threads.emplace_back(lane_loop, S, i);
  *out = S;
  return TG_OK;
}

int tg_serve_submit(tg_server* S, int n, const double* F, long long* request_id) {
  if (!S || !F || !request_id || n < 1 || n > 64) return TG_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->stop) return TG_ERR_ARG;
    tg_server::Req q;
    q.n = n;
    std::memcpy(q.F, F, 9 * sizeof(double));
    q.t_arrive = now_ms(S->t0);
    S->reqs.push_back(q);
    *request_id = (long long)S->reqs.size() - 1;
    S->ready.push_back(*request_id);
  }
  S->cv_work.notify_one();
  return TG_OK;
}

int tg_serve_poll(tg_server* S, long long id, double* P, int* status, double* latency_ms) {
  if (!S) return TG_ERR_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (id < 0 || id >= (long long)S->reqs.size()) return TG_ERR_ARG;
  const tg_server::Req& q = S->reqs[id];
  if (!q.done) return 1;  // pending
  if (P) std::memcpy(P, q.P, 9 * sizeof(double));
  if (status) *status = q.status;
  if (latency_ms) *latency_ms = q.t_finish - q.t_arrive;
  return TG_OK;
}

int tg_serve_wait(tg_server* S) {
  if (!S) return TG_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv_done.wait(lk, [&] { return S->completed == (long long)S->reqs.size(); });
  return TG_OK;
}

int tg_serve_stats(tg_server* S, double* out, int n) {
  if (!S || !out || n < 1) return TG_ERR_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  const double v[6] = {(double)S->batches,
                       S->batches ? (double)S->batched_requests / S->batches : 0.0,
                       (double)S->max_busy,
                       (double)S->retried,
                       S->predict_ms(1000.0),
                       (double)S->completed};
  for (int i = 0; i < n && i < 6; ++i) out[i] = v[i];
  return TG_OK;
}

const char* tg_serve_error(const tg_server* S) { return S ? S->err.c_str() : ""; }

int tg_serve_destroy(tg_server* S) {
  if (!S) return TG_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->threads) t.join();
  delete S;
  return TG_OK;
}

}  // extern "C"
