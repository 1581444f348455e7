// Device-resident Krylov solvers for the derivative operators.
//
// eigsolve: KrylovKit's Lanczos as MPSKit uses it through `fixedpoint`
// (src/algorithms/fixedpoint.jl:15-18): start from x0/|x0|, one matvec per expansion,
// full re-orthogonalisation (two classical Gram-Schmidt passes), diagonalise the
// projected matrix when the space is full, when beta <= tol, or after every step when
// `eager`; a Ritz pair is converged when |beta * U[K, i]| <= tol; thick restart keeps
// (3*krylovdim + 2)/5 Ritz vectors at most `maxiter` times.
//
// exponentiate: Lanczos approximation of exp(t H) x with time-step halving until the
// a-posteriori error estimate |beta_K c_K| |x| <= tol * tau (KrylovKit `exponentiate`,
// used by `integrate`, src/algorithms/timestep/integrators.jl:44-53).
//
// The Krylov basis, the work vector and all reductions stay in HBM in FP64; only the
// projected matrices (a few hundred numbers) visit the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "gb_common.h"

namespace gb {

void heff_apply_raw(gb_heff* h, const void* x, void* y);
int heff_precision(const gb_heff* h);

// Cyclic Jacobi eigen-decomposition of a small real symmetric matrix (row-major n x n).
// D ascending; U[:, j] (row-major U[i*n + j]) the eigenvector of D[j].
void sym_eig(int n, const std::vector<double>& Ain, std::vector<double>& D,
             std::vector<double>& U) {
  std::vector<double> A(Ain);
  U.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) U[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double a = A[i * n + j] * A[i * n + j];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double app = A[p * n + p], aqq = A[q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- J^T A J
          double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double ukp = U[k * n + p], ukq = U[k * n + q];
          U[k * n + p] = c * ukp - s * ukq;
          U[k * n + q] = s * ukp + c * ukq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
  D.resize(n);
  std::vector<double> U2((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    D[j] = A[idx[j] * n + idx[j]];
    for (int i = 0; i < n; ++i) U2[i * n + j] = U[i * n + idx[j]];
  }
  U.swap(U2);
}

struct KrylovWork {
  void* V = nullptr;  // (kd+1) vectors of n elements
  void* w = nullptr;
  void* tmp = nullptr;
};

static void orthogonalize(gb_ctx* ctx, int dtype, int64_t n, int k, void* V, void* w,
                          std::vector<cplx>& h) {
  std::vector<cplx> c(k), c2(k);
  multi_dot(ctx, dtype, n, k, V, n, w, c.data());
  std::vector<cplx> neg(k);
  for (int j = 0; j < k; ++j) neg[j] = cplx{-c[j].re, -c[j].im};
  multi_axpy(ctx, dtype, n, k, V, n, neg.data(), w);
  multi_dot(ctx, dtype, n, k, V, n, w, c2.data());
  for (int j = 0; j < k; ++j) neg[j] = cplx{-c2[j].re, -c2[j].im};
  multi_axpy(ctx, dtype, n, k, V, n, neg.data(), w);
  h.resize(k);
  for (int j = 0; j < k; ++j) h[j] = cplx{c[j].re + c2[j].re, c[j].im + c2[j].im};
}

// x <- sum_j coef[j] V[j]
static void combine(gb_ctx* ctx, int dtype, int64_t n, int k, const void* V,
                    const std::vector<cplx>& coef, void* x) {
  fill_zero(ctx, x, (size_t)n * elem_size(dtype));
  multi_axpy(ctx, dtype, n, k, V, n, coef.data(), x);
}

// The vector space of a solve: the dense vectors of the operator, or -- for a U(1)
// operator whose sectors are known -- only their charge-allowed entries (the rest of the
// charge-sorted embedding is exactly zero and stays so under H), which cuts the traffic of
// the re-orthogonalisation and of every vector operation by the sector fraction.
struct KrylovSpace {
  gb_heff* h;
  bool compact;
  int64_t n;  // length of the solver's vectors
  KrylovSpace(gb_heff* h_, int64_t dense_n) : h(h_) {
    HeffCompact c;
    compact = heff_compact(h, &c);
    n = compact ? c.n : dense_n;
  }
  void apply(const void* x, void* y) const {
    if (compact) heff_apply_compact(h, x, y);
    else heff_apply_raw(h, x, y);
  }
  // solver vector <- dense x, and back (the back copy zero-fills the rest of x)
  void load(gb_ctx* ctx, int dtype, const void* dense, void* v) const {
    if (compact) heff_gather(h, dense, v);
    else GB_CHECK_CUDA(cudaMemcpyAsync(v, dense, (size_t)n * elem_size(dtype),
                                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  void store(gb_ctx* ctx, int dtype, const void* v, void* dense) const {
    if (compact) heff_scatter(h, v, dense);
    else GB_CHECK_CUDA(cudaMemcpyAsync(dense, v, (size_t)n * elem_size(dtype),
                                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
};

int heff_eigsolve_raw(gb_ctx* ctx, gb_heff* h, int64_t n_dense, int dtype, void* x,
                      int krylovdim, int maxiter, double tol, bool eager, double* lambda,
                      gb_krylov_info* info) {
  GB_REQUIRE(krylovdim >= 1 && krylovdim <= 64 && maxiter >= 1, "eigsolve: krylovdim/maxiter");
  const KrylovSpace sp(h, n_dense);
  const int64_t n = sp.n;
  const size_t es = elem_size(dtype);
  const int kd = krylovdim;
  char* V = (char*)scratch(ctx, SLOT_KRYLOV, (size_t)(kd + 1) * n * es);
  void* w = scratch(ctx, SLOT_KRYLOV_W, (size_t)n * es);
  auto vec = [&](int j) { return (void*)(V + (size_t)j * n * es); };
  sp.load(ctx, dtype, x, vec(0));
  double nx = nrm2(ctx, dtype, n, vec(0));
  if (!std::isfinite(nx)) throw Error(GB_ERR_NAN, "eigsolve: initial vector is not finite");
  GB_REQUIRE(nx > 0, "eigsolve: initial vector has zero norm");
  scale(ctx, dtype, n, cplx{1.0 / nx, 0}, vec(0));
  const int howmany = 1;
  std::vector<double> H((size_t)(kd + 1) * (kd + 1), 0.0);  // row-major, stride kd+1
  const int LD = kd + 1;
  int K = 0, numops = 0, numiter = 1, converged = 0;
  double beta = 0.0;
  std::vector<double> D, U;
  std::vector<double> f;
  // With split-precision contractions the residual cannot fall below the operator's own
  // accuracy (~1e-6 relative); two restarts in a row that do not bring it 10% below the
  // best value so far end the solve (reported as not converged, as when maxiter runs out)
  // instead of spending the remaining restarts on rounding noise.  A single slow restart of
  // a hard problem does not.  FP64 operators keep KrylovKit's plain maxiter rule.
  const bool split = heff_precision(h) != GB_PREC_FP64;
  double best_res = INFINITY;
  int stalls = 0;
  while (true) {
    sp.apply(vec(K), w);
    ++numops;
    std::vector<cplx> hc;
    orthogonalize(ctx, dtype, n, K + 1, V, w, hc);
    for (int i = 0; i <= K; ++i) {
      H[i * LD + K] = hc[i].re;
      H[K * LD + i] = hc[i].re;
    }
    ++K;
    beta = nrm2(ctx, dtype, n, w);
    if (!std::isfinite(beta))
      throw Error(GB_ERR_NAN, "eigsolve: non-finite residual (NaN or Inf in the operator)");
    if (K == kd || beta <= tol || (eager && K >= howmany)) {
      std::vector<double> Hk((size_t)K * K);
      for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) Hk[i * K + j] = H[i * LD + j];
      sym_eig(K, Hk, D, U);
      f.assign(K, 0.0);
      for (int i = 0; i < K; ++i) f[i] = beta * U[(K - 1) * K + i];
      converged = 0;
      while (converged < K && std::fabs(f[converged]) <= tol) ++converged;
      if (converged >= howmany || beta <= tol) break;
    }
    if (K < kd) {
      GB_CHECK_CUDA(cudaMemcpyAsync(vec(K), w, n * es, cudaMemcpyDeviceToDevice, ctx->stream));
      scale(ctx, dtype, n, cplx{1.0 / beta, 0}, vec(K));
      continue;
    }
    if (numiter == maxiter) break;
    if (split) {
      const double res = std::fabs(f[0]);
      if (res > 0.9 * best_res) {
        if (++stalls >= 2) break;
      } else {
        stalls = 0;
      }
      best_res = std::min(best_res, res);
    }
    // thick restart: V[:keep] <- V[:K] U[:, :keep]
    int keep = (3 * kd + 2 * howmany) / 5;
    keep = std::max(1, std::min(keep, K - 1));
    void* tmp = scratch(ctx, SLOT_TMP, (size_t)keep * n * es);
    for (int j = 0; j < keep; ++j) {
      std::vector<cplx> coef(K);
      for (int i = 0; i < K; ++i) coef[i] = cplx{U[i * K + j], 0.0};
      combine(ctx, dtype, n, K, V, coef, (char*)tmp + (size_t)j * n * es);
    }
    GB_CHECK_CUDA(cudaMemcpyAsync(V, tmp, (size_t)keep * n * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    std::fill(H.begin(), H.end(), 0.0);
    for (int j = 0; j < keep; ++j) {
      H[j * LD + j] = D[j];
      H[keep * LD + j] = f[j];
      H[j * LD + keep] = f[j];
    }
    GB_CHECK_CUDA(cudaMemcpyAsync(vec(keep), w, n * es, cudaMemcpyDeviceToDevice, ctx->stream));
    scale(ctx, dtype, n, cplx{1.0 / beta, 0}, vec(keep));
    K = keep;
    ++numiter;
  }
  std::vector<cplx> coef(K);
  for (int i = 0; i < K; ++i) coef[i] = cplx{U[i * K + 0], 0.0};
  combine(ctx, dtype, n, K, V, coef, w);
  double nn = nrm2(ctx, dtype, n, w);
  scale(ctx, dtype, n, cplx{1.0 / nn, 0}, w);
  sp.store(ctx, dtype, w, x);
  *lambda = D[0];
  if (info) {
    info->converged = converged;
    info->numops = numops;
    info->numiter = numiter;
    info->normres = std::fabs(f[0]);
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB_OK;
}

int heff_exponentiate_raw(gb_ctx* ctx, gb_heff* h, int64_t n_dense, int dtype, void* x_dense,
                          double t_re, double t_im, int krylovdim, int maxiter, double tol,
                          gb_krylov_info* info) {
  GB_REQUIRE(krylovdim >= 1 && krylovdim <= 64, "exponentiate: krylovdim");
  GB_REQUIRE(is_cplx(dtype) || t_im == 0.0, "exponentiate: complex time needs complex storage");
  const KrylovSpace sp(h, n_dense);
  const int64_t n = sp.n;
  // the evolving state in the solver's space (compact: an operator-owned vector)
  void* x = x_dense;
  if (sp.compact) {
    HeffCompact c;
    heff_compact(h, &c);
    x = c.xcomp;
    sp.load(ctx, dtype, x_dense, x);
  }
  const size_t es = elem_size(dtype);
  const int kd = krylovdim;
  char* V = (char*)scratch(ctx, SLOT_KRYLOV, (size_t)(kd + 1) * n * es);
  void* w = scratch(ctx, SLOT_KRYLOV_W, (size_t)n * es);
  auto vec = [&](int j) { return (void*)(V + (size_t)j * n * es); };
  const std::complex<double> total(t_re, t_im);
  double tau_left = 1.0, tau = 1.0;
  int numops = 0, numiter = 0;
  const int maxsteps = std::max(1, maxiter) * 50;
  while (tau_left > 0 && numiter < maxsteps) {
    ++numiter;
    double nrm = nrm2(ctx, dtype, n, x);
    if (nrm == 0.0) break;
    GB_CHECK_CUDA(cudaMemcpyAsync(vec(0), x, n * es, cudaMemcpyDeviceToDevice, ctx->stream));
    scale(ctx, dtype, n, cplx{1.0 / nrm, 0}, vec(0));
    std::vector<double> alphas, betas;
    int K = 0;
    bool happy = false;
    for (int j = 0; j < kd; ++j) {
      sp.apply(vec(j), w);
      ++numops;
      std::vector<cplx> hc;
      orthogonalize(ctx, dtype, n, j + 1, V, w, hc);
      double a = hc[j].re;
      double b = nrm2(ctx, dtype, n, w);
      alphas.push_back(a);
      betas.push_back(b);
      K = j + 1;
      if (b <= tol * 1e-3) {
        happy = true;
        break;
      }
      if (j + 1 < kd + 1) {
        GB_CHECK_CUDA(cudaMemcpyAsync(vec(j + 1), w, n * es, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        scale(ctx, dtype, n, cplx{1.0 / b, 0}, vec(j + 1));
      }
    }
    std::vector<double> T((size_t)K * K, 0.0), D, U;
    for (int i = 0; i < K; ++i) {
      T[i * K + i] = alphas[i];
      if (i + 1 < K) T[i * K + i + 1] = T[(i + 1) * K + i] = betas[i];
    }
    sym_eig(K, T, D, U);
    tau = std::min(tau, tau_left);
    std::vector<std::complex<double>> c(K);
    while (true) {
      for (int i = 0; i < K; ++i) {
        std::complex<double> acc = 0.0;
        for (int j = 0; j < K; ++j) acc += U[i * K + j] * std::exp(total * tau * D[j]) * U[0 * K + j];
        c[i] = acc;
      }
      double err = happy ? 0.0 : std::abs(betas[K - 1] * c[K - 1]) * nrm;
      if (err <= tol * tau || tau < 1e-12) break;
      tau *= 0.5;
    }
    std::vector<cplx> coef(K);
    for (int i = 0; i < K; ++i) coef[i] = cplx{nrm * c[i].real(), nrm * c[i].imag()};
    if (!is_cplx(dtype))
      for (auto& q : coef) q.im = 0.0;
    combine(ctx, dtype, n, K, V, coef, x);
    tau_left -= tau;
    if (tau_left < 1e-15) tau_left = 0.0;
    tau = std::min(2 * tau, 1.0);
  }
  if (sp.compact) sp.store(ctx, dtype, x, x_dense);
  if (info) {
    info->converged = tau_left == 0.0 ? 1 : 0;
    info->numops = numops;
    info->numiter = numiter;
    info->normres = 0.0;
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB_OK;
}


// ------------------------------------------------------------------ environment linsolve
// x - T(x) = b on one level of an infinite environment (KrylovKit linsolve(T, b, x0,
// GMRES(krylovdim, maxiter, tol), 1, -1) as compute_leftenvs!/compute_rightenvs! call it,
// src/environments/infinite_envs.jl:236, 252, 307, 322): T(v) = transfer(v, W, A, A) (left
// or right), followed, when lvec is given, by the regularisation v_c -= tr(lvec v_c) rvec on
// every channel c (the identity levels).  Restarted GMRES with Givens rotations on the host;
// the Krylov vectors stay on the device and are orthogonalised in two batched CGS passes.
// With a split-precision transfer a restart that reduces the true residual by less than 10%
// ends the solve (the operator is accurate to ~1e-6; see heff_eigsolve_raw).
int env_linsolve_raw(gb_ctx* ctx, int side, const gb_tensor* W, const gb_tensor* A, int prec,
                     const gb_tensor* lvec, const gb_tensor* rvec, const gb_tensor* b,
                     gb_tensor* x, int krylovdim, int maxiter, double tol, gb_krylov_info* info) {
  using zc = std::complex<double>;
  const int dt = b->dtype;
  const size_t es = elem_size(dt);
  int64_t n = 1;
  for (int i = 0; i < b->ndim; ++i) n *= b->dims[i];
  const int kd = std::max(1, std::min(krylovdim, 64));
  char* V = (char*)scratch(ctx, SLOT_KRYLOV, (size_t)(kd + 2) * n * es);
  void* w = scratch(ctx, SLOT_KRYLOV_W, (size_t)n * es);
  auto vec = [&](int j) { return (void*)(V + (size_t)j * n * es); };
  void* Tv = vec(kd + 1);
  auto wrap = [&](void* p) {
    gb_tensor t;
    t.ctx = ctx;
    t.kind = b->kind;
    t.dtype = dt;
    t.ndim = b->ndim;
    for (int i = 0; i < 6; ++i) t.dims[i] = b->dims[i];
    t.data = p;
    t.bytes = (size_t)n * es;
    return t;
  };
  auto check = [](int rc) {
    if (rc != GB_OK) throw Error(rc, gb_last_error());
  };
  int numops = 0;
  // out <- v - T(v)
  auto apply = [&](const void* v, void* out) {
    gb_tensor tin = wrap((void*)v), tout = wrap(Tv);
    if (side == 0)
      check(gb_env_transfer_left(ctx, &tin, W, A, A, prec, &tout));
    else
      check(gb_env_transfer_right(ctx, &tin, W, A, A, prec, &tout));
    if (lvec)
      for (int64_t c = 0; c < b->dims[1]; ++c) check(gb_env_regularize(ctx, &tout, c, lvec, rvec));
    GB_CHECK_CUDA(cudaMemcpyAsync(out, v, (size_t)n * es, cudaMemcpyDeviceToDevice, ctx->stream));
    axpy(ctx, dt, n, cplx{-1.0, 0.0}, Tv, out);
    ++numops;
  };
  const bool split = prec != GB_PREC_FP64;
  const bool cx = is_cplx(dt);
  double res = INFINITY, last = INFINITY;
  int it = 0, converged = 0;
  for (it = 0; it < std::max(1, maxiter); ++it) {
    // r = b - (x - T x)
    apply(x->data, w);
    axpy(ctx, dt, n, cplx{-1.0, 0.0}, b->data, w);  // w = (x - T x) - b
    const double beta = nrm2(ctx, dt, n, w);
    res = beta;
    if (beta <= tol) {
      converged = 1;
      break;
    }
    if (split && beta > 0.9 * last) break;
    last = beta;
    GB_CHECK_CUDA(cudaMemcpyAsync(vec(0), w, (size_t)n * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    scale(ctx, dt, n, cplx{-1.0 / beta, 0.0}, vec(0));  // V0 = r / beta
    std::vector<std::vector<zc>> R;                       // rotated Hessenberg columns
    std::vector<double> cs;
    std::vector<zc> sn, g(1, zc(beta, 0.0));
    int k = 0;
    for (int j = 0; j < kd; ++j) {
      apply(vec(j), w);
      std::vector<cplx> hc;
      orthogonalize(ctx, dt, n, j + 1, V, w, hc);
      const double hn = nrm2(ctx, dt, n, w);
      std::vector<zc> h(j + 2);
      for (int i = 0; i <= j; ++i) h[i] = zc(hc[i].re, cx ? hc[i].im : 0.0);
      h[j + 1] = zc(hn, 0.0);
      for (int i = 0; i < j; ++i) {  // previous rotations
        const zc t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -std::conj(sn[i]) * h[i] + cs[i] * h[i + 1];
        h[i] = t;
      }
      const double a = std::abs(h[j]);
      double c;
      zc s;
      if (a == 0.0) {
        c = 0.0;
        s = zc(1.0, 0.0);
        h[j] = h[j + 1];
      } else {
        const double r = std::hypot(a, hn);
        c = a / r;
        s = (h[j] / a) * (hn / r);
        h[j] = (h[j] / a) * r;
      }
      h[j + 1] = 0.0;
      cs.push_back(c);
      sn.push_back(s);
      g.push_back(-std::conj(s) * g[j]);
      g[j] = c * g[j];
      R.push_back(h);
      k = j + 1;
      res = std::abs(g[j + 1]);
      if (res <= tol || hn < 1e-300) break;
      if (j + 1 < kd) {
        GB_CHECK_CUDA(cudaMemcpyAsync(vec(j + 1), w, (size_t)n * es, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        scale(ctx, dt, n, cplx{1.0 / hn, 0.0}, vec(j + 1));
      }
    }
    // R y = g (upper triangular, columns R[j][0..j]); x += sum_i y_i V_i
    std::vector<zc> y(k);
    for (int i = k - 1; i >= 0; --i) {
      zc acc = g[i];
      for (int jj = i + 1; jj < k; ++jj) acc -= R[jj][i] * y[jj];
      y[i] = acc / R[i][i];
    }
    std::vector<cplx> coef(k);
    for (int i = 0; i < k; ++i) coef[i] = cplx{y[i].real(), cx ? y[i].imag() : 0.0};
    multi_axpy(ctx, dt, n, k, V, n, coef.data(), x->data);
  }
  if (!converged && it >= std::max(1, maxiter)) {
    // report the true residual of the final iterate
    apply(x->data, w);
    axpy(ctx, dt, n, cplx{-1.0, 0.0}, b->data, w);
    res = nrm2(ctx, dt, n, w);
    converged = res <= tol;
  }
  if (info) {
    info->converged = converged;
    info->numops = numops;
    info->numiter = it;
    info->normres = res;
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB_OK;
}

}  // namespace gb
