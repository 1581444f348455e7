// C ABI of libmpsgb (declared in include/mpsgb.h): contexts, tensors with layout
// conversion at the boundary, BLAS-1, environment transfers, state helpers and the
// gauge factorisations.  Every entry point converts exceptions into status codes.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <numeric>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <thread>

#include "gb_common.h"

namespace gb {

static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }

void* scratch(gb_ctx* ctx, int slot, size_t bytes) {
  Scratch& s = ctx->scratch[slot];
  if (s.bytes >= bytes && s.ptr) return s.ptr;
  if (s.ptr) {
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(s.ptr);
    s.ptr = nullptr;
    s.bytes = 0;
  }
  size_t nb = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(&s.ptr, nb);
  if (e != cudaSuccess) {
    s.ptr = nullptr;
    throw Error(GB_ERR_OOM, std::string("scratch cudaMalloc: ") + cudaGetErrorString(e));
  }
  s.bytes = nb;
  return s.ptr;
}

// source sites of traced launches ("file.cu:line"), shared by every context
static std::mutex g_site_mu;
static std::vector<std::string> g_site_names;
static std::map<std::pair<const char*, int>, int> g_site_ids;

void trace_point(gb_ctx* ctx, const char* file, int line) {
  int id;
  {
    std::lock_guard<std::mutex> lk(g_site_mu);
    auto it = g_site_ids.find({file, line});
    if (it == g_site_ids.end()) {
      std::string f(file);
      size_t sl = f.find_last_of('/');
      if (sl != std::string::npos) f = f.substr(sl + 1);
      id = (int)g_site_names.size();
      g_site_names.push_back(f + ":" + std::to_string(line));
      g_site_ids.emplace(std::make_pair(file, line), id);
    } else {
      id = it->second;
    }
  }
  if (ctx->trace_used == ctx->trace_ev.size()) {
    cudaEvent_t e;
    GB_CHECK_CUDA(cudaEventCreate(&e));
    ctx->trace_ev.push_back(e);
    ctx->trace_site.push_back(-1);
  }
  GB_CHECK_CUDA(cudaEventRecord(ctx->trace_ev[ctx->trace_used], ctx->stream));
  ctx->trace_site[ctx->trace_used++] = id;
}

gb_heff* heff_build(gb_ctx* ctx, int kind, const gb_tensor* GL, const gb_tensor* W1,
                    const gb_tensor* W2, const gb_tensor* GR, int prec);
void heff_free(gb_heff* h);
void heff_set_precision(gb_heff* h, int prec);
void heff_set_sectors(gb_heff* h, const int32_t* ql, const int32_t* qp1, const int32_t* qp2,
                      const int32_t* qr);
void heff_apply_raw(gb_heff* h, const void* x, void* y);
int env_linsolve_raw(gb_ctx* ctx, int side, const gb_tensor* W, const gb_tensor* A, int prec,
                     const gb_tensor* lvec, const gb_tensor* rvec, const gb_tensor* b,
                     gb_tensor* x, int krylovdim, int maxiter, double tol, gb_krylov_info* info);
int heff_eigsolve_raw(gb_ctx* ctx, gb_heff* h, int64_t n, int dtype, void* x, int krylovdim,
                      int maxiter, double tol, bool eager, double* lambda, gb_krylov_info* info);
int heff_exponentiate_raw(gb_ctx* ctx, gb_heff* h, int64_t n, int dtype, void* x, double t_re,
                          double t_im, int krylovdim, int maxiter, double tol,
                          gb_krylov_info* info);

}  // namespace gb

// gb_heff is opaque here; these accessors live in heff_access below
struct gb_heff;
namespace gb {
struct HeffInfo {
  gb_ctx* ctx;
  int kind, dtype, prec, xndim;
  int64_t xdims[4];
  int64_t xnumel;
  double flops;
  const char* terms;
};
HeffInfo heff_info(const gb_heff* h);
std::string heff_describe(const gb_heff* h);
}  // namespace gb

using namespace gb;

#define API_BEGIN try {
#define API_END                                 \
  }                                             \
  catch (const gb::Error& e) {                  \
    gb::set_last_error(e.what());               \
    return e.code;                              \
  }                                             \
  catch (const std::exception& e) {             \
    gb::set_last_error(e.what());               \
    return GB_ERR_CUDA;                         \
  }                                             \
  catch (...) {                                 \
    gb::set_last_error("unknown error");        \
    return GB_ERR_CUDA;                         \
  }                                             \
  return GB_OK;

namespace {

struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DevGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// device-layout strides of a tensor expressed over the reference leg order
void ref_strides(int kind, int ndim, const int64_t* dims, int64_t* ref, int64_t* dev) {
  // reference: plain column-major over dims
  int64_t s = 1;
  for (int i = 0; i < ndim; ++i) {
    ref[i] = s;
    s *= dims[i];
  }
  for (int i = 0; i < ndim; ++i) dev[i] = ref[i];
  if (kind == GB_KIND_AC2) {  // ref (l, s1, r, s2) -> dev (l, s1, s2, r)
    dev[0] = 1;
    dev[1] = dims[0];
    dev[3] = dims[0] * dims[1];
    dev[2] = dims[0] * dims[1] * dims[3];
  } else if (kind == GB_KIND_GL) {  // ref (a, w, a') -> dev (a, a', w)
    dev[0] = 1;
    dev[2] = dims[0];
    dev[1] = dims[0] * dims[2];
  }
}

bool needs_permute(int kind) { return kind == GB_KIND_AC2 || kind == GB_KIND_GL; }

gb_tensor* new_tensor(gb_ctx* ctx, int kind, int dtype, int ndim, const int64_t* dims) {
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(dtype == GB_F64 || dtype == GB_C128, "dtype must be GB_F64 or GB_C128");
  GB_REQUIRE(ndim >= 1 && ndim <= 6, "ndim must be in 1..6");
  int want = -1;
  switch (kind) {
    case GB_KIND_MPS: want = 3; break;
    case GB_KIND_BOND: want = 2; break;
    case GB_KIND_AC2: want = 4; break;
    case GB_KIND_GL: want = 3; break;
    case GB_KIND_GR: want = 3; break;
    case GB_KIND_MPO: want = 4; break;
    case GB_KIND_GENERIC: break;
    default: throw Error(GB_ERR_ARG, "unknown tensor kind");
  }
  GB_REQUIRE(want < 0 || ndim == want, "tensor rank does not match its kind");
  for (int i = 0; i < ndim; ++i) GB_REQUIRE(dims[i] >= 0, "negative dimension");
  gb_tensor* t = new gb_tensor();
  t->ctx = ctx;
  t->kind = kind;
  t->dtype = dtype;
  t->ndim = ndim;
  for (int i = 0; i < ndim; ++i) t->dims[i] = dims[i];
  t->bytes = (size_t)numel(t) * elem_size(dtype);
  if (t->bytes) {
    cudaError_t e = cudaMallocAsync(&t->data, t->bytes, ctx->stream);
    if (e != cudaSuccess) {
      delete t;
      throw Error(GB_ERR_OOM, std::string("tensor allocation: ") + cudaGetErrorString(e));
    }
  }
  if (kind == GB_KIND_MPO) t->host_mpo.assign(numel(t) * (is_cplx(dtype) ? 2 : 1), 0.0);
  return t;
}

void free_tensor(gb_tensor* t) {
  if (!t) return;
  if (t->data) cudaFreeAsync(t->data, t->ctx->stream);
  delete t;
}

// ------------------------------------------------------------------ small kernels
__global__ void conj_transpose_kernel(int64_t m, int64_t n, const double* __restrict__ A,
                                      int64_t lda, double* __restrict__ B, int64_t ldb, int cx,
                                      int conj) {
  __shared__ double tr[32][33], ti[32][33];
  int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    int64_t i = i0 + threadIdx.x, j = j0 + k;
    double re = 0, im = 0;
    if (i < m && j < n) {
      if (cx) {
        re = A[2 * (i + lda * j)];
        im = A[2 * (i + lda * j) + 1];
      } else {
        re = A[i + lda * j];
      }
    }
    tr[k][threadIdx.x] = re;
    ti[k][threadIdx.x] = conj ? -im : im;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    int64_t j = j0 + threadIdx.x, i = i0 + k;  // B[j, i] = A[i, j]
    if (i < m && j < n) {
      if (cx) {
        B[2 * (j + ldb * i)] = tr[threadIdx.x][k];
        B[2 * (j + ldb * i) + 1] = ti[threadIdx.x][k];
      } else {
        B[j + ldb * i] = tr[threadIdx.x][k];
      }
    }
  }
}

void conj_transpose(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda,
                    void* B, int64_t ldb) {
  if (m == 0 || n == 0) return;
  dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
  conj_transpose_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>(
      m, n, (const double*)A, lda, (double*)B, ldb, is_cplx(dtype), 1);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

// R (k x n) upper part of QR output A (lda), zero below the diagonal
__global__ void extract_upper_kernel(int64_t k, int64_t n, const double* __restrict__ A,
                                     int64_t lda, double* __restrict__ R, int cx) {
  int64_t tot = k * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % k, j = e / k;
    bool up = i <= j;
    if (cx) {
      R[2 * e] = up ? A[2 * (i + lda * j)] : 0.0;
      R[2 * e + 1] = up ? A[2 * (i + lda * j) + 1] : 0.0;
    } else {
      R[e] = up ? A[i + lda * j] : 0.0;
    }
  }
}

// make diag(R) real non-negative: Q[:, j] *= ph_j, R[j, :] *= conj(ph_j)
__global__ void fix_phase_kernel(int64_t m, int64_t k, int64_t n, double* __restrict__ Q,
                                 int64_t ldq, double* __restrict__ R, int64_t ldr, int cx) {
  int64_t j = blockIdx.x;
  if (j >= k) return;
  double pr, pi;
  if (cx) {
    double a = R[2 * (j + ldr * j)], b = R[2 * (j + ldr * j) + 1];
    double r = hypot(a, b);
    pr = r > 0 ? a / r : 1.0;
    pi = r > 0 ? b / r : 0.0;
  } else {
    double a = R[j + ldr * j];
    pr = a < 0 ? -1.0 : 1.0;
    pi = 0.0;
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    if (cx) {
      double a = Q[2 * (i + ldq * j)], b = Q[2 * (i + ldq * j) + 1];
      Q[2 * (i + ldq * j)] = a * pr - b * pi;
      Q[2 * (i + ldq * j) + 1] = a * pi + b * pr;
    } else {
      Q[i + ldq * j] *= pr;
    }
  }
  for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
    if (cx) {  // times conj(ph)
      double a = R[2 * (j + ldr * c)], b = R[2 * (j + ldr * c) + 1];
      R[2 * (j + ldr * c)] = a * pr + b * pi;
      R[2 * (j + ldr * c) + 1] = b * pr - a * pi;
    } else {
      R[j + ldr * c] *= pr;
    }
  }
}

// S (k reals) -> diagonal k x k matrix of dtype, scaled by s
__global__ void diag_kernel(int64_t k, const double* __restrict__ S, double scl,
                            double* __restrict__ out, int cx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % k, j = e / k;
    double v = (i == j) ? S[i] * scl : 0.0;
    if (cx) {
      out[2 * e] = v;
      out[2 * e + 1] = 0.0;
    } else {
      out[e] = v;
    }
  }
}

cusolverDnHandle_t solver(gb_ctx* ctx) {
  if (!ctx->solver) {
    cusolverDnHandle_t h;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS)
      throw Error(GB_ERR_CUDA, "cusolverDnCreate failed");
    cusolverDnSetStream(h, ctx->stream);
    cusolverDnParams_t p;
    cusolverDnCreateParams(&p);
    ctx->solver = h;
    ctx->solver_params = p;
  }
  return (cusolverDnHandle_t)ctx->solver;
}

#define CUSOLVER_CHECK(x)                                                         \
  do {                                                                            \
    cusolverStatus_t _s = (x);                                                    \
    if (_s != CUSOLVER_STATUS_SUCCESS)                                            \
      throw Error(GB_ERR_CUDA, std::string(#x) + " failed: " + std::to_string(_s)); \
  } while (0)

__global__ void scale_columns_kernel(int64_t m, int64_t n, double* __restrict__ U,
                                     const double* __restrict__ S, int cx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = e / m;
    double sj = S[j];
    double f = sj > 0 ? 1.0 / sj : 0.0;
    if (cx) {
      U[2 * e] *= f;
      U[2 * e + 1] *= f;
    } else {
      U[e] *= f;
    }
  }
}

// sigma_j = sqrt(max(lambda_{n-1-j}, 0)): eigenvalues ascending -> singular values descending
__global__ void sqrt_reverse_kernel(int64_t n, const double* __restrict__ lam,
                                    double* __restrict__ S) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    double v = lam[n - 1 - j];
    S[j] = v > 0 ? sqrt(v) : 0.0;
  }
}

void qr_pos(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* M, void* Q, void* R);

// economy SVD of M (m x n, m >= n), col-major lda = m: U (m x n), S (n, descending), VT (n x n)
void svd_tall(gb_ctx* ctx, int dtype, int64_t m, int64_t n, void* A, void* U, double* S,
              void* VT) {
  cusolverDnHandle_t h = solver(ctx);
  cudaDataType t = is_cplx(dtype) ? CUDA_C_64F : CUDA_R_64F;
  const size_t es = elem_size(dtype);
  size_t dws = 0, hws = 0;
  if (ctx->svd_method == GB_SVD_GESVDP) {
    // V (n x n) into the first part of a scratch slot, then VT = V^H
    char* V = (char*)scratch(ctx, SLOT_TMP2, (size_t)n * n * es + 256);
    CUSOLVER_CHECK(cusolverDnXgesvdp_bufferSize(h, (cusolverDnParams_t)ctx->solver_params,
                                                CUSOLVER_EIG_MODE_VECTOR, 1, m, n, t, A, m,
                                                CUDA_R_64F, S, t, U, m, t, V, n, t, &dws, &hws));
    char* dw = (char*)scratch(ctx, SLOT_TMP, dws + 512);
    int* dinfo = (int*)(dw + ((dws + 255) & ~size_t(255)));
    std::vector<char> hw(hws + 1);
    double herr = 0.0;
    CUSOLVER_CHECK(cusolverDnXgesvdp(h, (cusolverDnParams_t)ctx->solver_params,
                                     CUSOLVER_EIG_MODE_VECTOR, 1, m, n, t, A, m, CUDA_R_64F, S, t,
                                     U, m, t, V, n, t, dw, dws, hw.data(), hws, dinfo, &herr));
    GB_TRACE(ctx);
    count_launch(ctx);
    int hinfo = 0;
    GB_CHECK_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hinfo != 0) throw Error(GB_ERR_CUDA, "gesvdp info = " + std::to_string(hinfo));
    conj_transpose(ctx, dtype, n, n, V, n, VT, n);
    return;
  }
  CUSOLVER_CHECK(cusolverDnXgesvd_bufferSize(h, (cusolverDnParams_t)ctx->solver_params, 'S', 'S',
                                             m, n, t, A, m, CUDA_R_64F, S, t, U, m, t, VT, n, t,
                                             &dws, &hws));
  void* dw = scratch(ctx, SLOT_TMP, dws + 256);
  std::vector<char> hw(hws + 1);
  int* dinfo = (int*)((char*)dw + ((dws + 127) & ~size_t(127)));
  CUSOLVER_CHECK(cusolverDnXgesvd(h, (cusolverDnParams_t)ctx->solver_params, 'S', 'S', m, n, t,
                                  A, m, CUDA_R_64F, S, t, U, m, t, VT, n, t, dw, dws, hw.data(),
                                  hws, dinfo));
  GB_TRACE(ctx);
  int hinfo = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  count_launch(ctx);
  if (hinfo != 0) throw Error(GB_ERR_CUDA, "gesvd info = " + std::to_string(hinfo));
}

__global__ void scale_rows_kernel(int64_t m, int64_t n, double* __restrict__ A, int64_t lda,
                                  const double* __restrict__ S, int cx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % m, j = e / m;
    double f = S[i];
    if (cx) {
      A[2 * (i + lda * j)] *= f;
      A[2 * (i + lda * j) + 1] *= f;
    } else {
      A[i + lda * j] *= f;
    }
  }
}

__global__ void inv_kernel(int64_t n, const double* __restrict__ S, double* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x)
    out[j] = S[j] > 0 ? 1.0 / S[j] : 0.0;
}

// positive QR of M (m x n): Q (m x k), R (k x n), k = min(m, n)
void qr_pos(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* M, void* Q, void* R) {
  cusolverDnHandle_t h = solver(ctx);
  const bool cx = is_cplx(dtype);
  cudaDataType t = cx ? CUDA_C_64F : CUDA_R_64F;
  const size_t es = elem_size(dtype);
  int64_t k = std::min(m, n);
  int64_t ncols = std::max(n, k);
  // work matrix: m x n copy of M (plus room for orgqr on the first k columns)
  char* A = (char*)scratch(ctx, SLOT_GAUGE, (size_t)m * ncols * es + 256);
  GB_CHECK_CUDA(cudaMemcpyAsync(A, M, (size_t)m * n * es, cudaMemcpyDeviceToDevice, ctx->stream));
  char* tau = (char*)scratch(ctx, SLOT_GAUGE3, (size_t)k * es + 256);
  size_t dws = 0, hws = 0;
  CUSOLVER_CHECK(cusolverDnXgeqrf_bufferSize(h, (cusolverDnParams_t)ctx->solver_params, m, n, t,
                                             A, m, t, tau, t, &dws, &hws));
  char* dw = (char*)scratch(ctx, SLOT_TMP, dws + 256);
  int* dinfo = (int*)scratch(ctx, SLOT_TMP2, 256);
  std::vector<char> hw(hws + 1);
  CUSOLVER_CHECK(cusolverDnXgeqrf(h, (cusolverDnParams_t)ctx->solver_params, m, n, t, A, m, t,
                                  tau, t, dw, dws, hw.data(), hws, dinfo));
  GB_TRACE(ctx);
  count_launch(ctx);
  // R = upper(A[:k, :])
  extract_upper_kernel<<<256, 256, 0, ctx->stream>>>(k, n, (const double*)A, m, (double*)R, cx);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  // Q from the reflectors (first k columns)
  int lwork = 0;
  if (cx) {
    CUSOLVER_CHECK(cusolverDnZungqr_bufferSize(h, (int)m, (int)k, (int)k, (cuDoubleComplex*)A,
                                               (int)m, (cuDoubleComplex*)tau, &lwork));
    char* wk = (char*)scratch(ctx, SLOT_TMP, (size_t)lwork * es + 256);
    CUSOLVER_CHECK(cusolverDnZungqr(h, (int)m, (int)k, (int)k, (cuDoubleComplex*)A, (int)m,
                                    (cuDoubleComplex*)tau, (cuDoubleComplex*)wk, lwork, dinfo));
    GB_TRACE(ctx);
  } else {
    CUSOLVER_CHECK(cusolverDnDorgqr_bufferSize(h, (int)m, (int)k, (int)k, (double*)A, (int)m,
                                               (double*)tau, &lwork));
    char* wk = (char*)scratch(ctx, SLOT_TMP, (size_t)lwork * es + 256);
    CUSOLVER_CHECK(cusolverDnDorgqr(h, (int)m, (int)k, (int)k, (double*)A, (int)m, (double*)tau,
                                    (double*)wk, lwork, dinfo));
    GB_TRACE(ctx);
  }
  count_launch(ctx);
  GB_CHECK_CUDA(cudaMemcpyAsync(Q, A, (size_t)m * k * es, cudaMemcpyDeviceToDevice, ctx->stream));
  fix_phase_kernel<<<(unsigned)k, 256, 0, ctx->stream>>>(m, k, n, (double*)Q, m, (double*)R, k,
                                                         cx);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  int hinfo = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hinfo != 0) throw Error(GB_ERR_CUDA, "QR info = " + std::to_string(hinfo));
}


// Truncated factorisation M ~ AL C AR through the eigendecomposition of the Gram matrix of
// the smaller side (FP64 syevd).  The Gram eigenvectors give one exactly isometric factor;
// the other factor (M V / sigma, or sigma^-1 U^H M) is made exactly isometric by a positive
// QR / LQ, whose triangular factor is absorbed into the bond matrix C = R Sigma (or Sigma L).
// The state AL C AR equals U Sigma V^H of the truncated SVD; C is triangular, not diagonal.
// Singular values from Gram eigenvalues carry an absolute error of about eps_mach * s_max^2 /
// s, so values below GRAM_FLOOR * s_max are rounding noise: when a kept value or the first
// discarded one lies below that floor, the rank and the discarded weight cannot be decided
// from them, and the function returns false without output (the caller then runs the SVD).
constexpr double GRAM_FLOOR = 1e-7;
bool svd_trunc_gram(gb_ctx* ctx, const gb_tensor* AC2, int64_t maxdim, double atol, int normalize,
                    gb_tensor** AL, gb_tensor** S, gb_tensor** AR, double* eps) {
  cusolverDnHandle_t h = solver(ctx);
  const int dt = AC2->dtype;
  const bool cx = is_cplx(dt);
  cudaDataType t = cx ? CUDA_C_64F : CUDA_R_64F;
  const size_t es = elem_size(dt);
  const int64_t Dl = AC2->dims[0], d1 = AC2->dims[1], Dr = AC2->dims[2], d2 = AC2->dims[3];
  const int64_t m = Dl * d1, n = d2 * Dr;
  const bool tall = m >= n;
  const int64_t g = tall ? n : m;
  const void* M = AC2->data;
  char* G = (char*)scratch(ctx, SLOT_GAUGE, (size_t)g * g * es + 256);
  if (tall)
    gemm_fp64(ctx, dt, 'C', 'N', n, n, m, cplx{1, 0}, M, m, 0, M, m, 0, cplx{0, 0}, G, n, 0, 1);
  else
    gemm_fp64(ctx, dt, 'N', 'C', m, m, n, cplx{1, 0}, M, m, 0, M, m, 0, cplx{0, 0}, G, m, 0, 1);
  double* lam = (double*)scratch(ctx, SLOT_KRYLOV_W, sizeof(double) * (2 * g + 64) + 4096);
  double* sig = lam + g + 32;
  (void)h;
  (void)t;
  int* dinfo = (int*)scratch(ctx, SLOT_TMP2, 256);
  sym_eig(ctx, dt, g, G, lam, dinfo);
  GB_TRACE(ctx);
  sqrt_reverse_kernel<<<64, 256, 0, ctx->stream>>>(g, lam, sig);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  std::vector<double> hs(g);
  int hinfo = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(hs.data(), sig, sizeof(double) * g, cudaMemcpyDeviceToHost,
                                ctx->stream));
  GB_CHECK_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hinfo != 0) throw Error(GB_ERR_CUDA, "syevd info = " + std::to_string(hinfo));
  int64_t keep = 0;
  for (int64_t i = 0; i < g; ++i)
    if (hs[i] > atol) ++keep;
  if (maxdim > 0) keep = std::min(keep, maxdim);
  keep = std::max<int64_t>(keep, 1);
  const double floor = GRAM_FLOOR * hs[0];
  if (!(hs[keep - 1] >= floor && (keep == g || hs[keep] >= floor))) return false;
  double e2 = 0.0;
  for (int64_t i = keep; i < g; ++i) e2 += hs[i] * hs[i];
  if (eps) *eps = std::sqrt(e2);
  GB_REQUIRE(hs[keep - 1] > 0.0, "svd_trunc (Gram): a kept singular value is zero");
  // E = eigenvectors of the kept singular values, descending: E[:, j] = G[:, g-1-j]
  char* E = (char*)scratch(ctx, SLOT_GAUGE2, (size_t)g * keep * es + 256);
  {
    int64_t dims[2] = {g, keep}, ins[2] = {1, -g}, outs[2] = {1, g};
    permute(ctx, dt, 2, dims, G + (size_t)(g - 1) * g * es, ins, E, outs);
  }
  double* isig = lam;  // lam no longer needed
  inv_kernel<<<32, 256, 0, ctx->stream>>>(keep, sig, isig);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  int64_t dl[3] = {Dl, d1, keep}, dr[3] = {keep, d2, Dr}, dc[2] = {keep, keep};
  gb_tensor* al = new_tensor(ctx, GB_KIND_MPS, dt, 3, dl);
  gb_tensor* ar = new_tensor(ctx, GB_KIND_MPS, dt, 3, dr);
  gb_tensor* cc = new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  char* F = (char*)scratch(ctx, SLOT_T1, (size_t)std::max(m, n) * keep * es + 256);
  if (tall) {
    // U_k = M E / sigma (m x keep) -> positive QR: U_k = Q R; AL = Q, C = R Sigma
    gemm_fp64(ctx, dt, 'N', 'N', m, keep, n, cplx{1, 0}, M, m, 0, E, n, 0, cplx{0, 0}, F, m, 0, 1);
    scale_columns_kernel<<<256, 256, 0, ctx->stream>>>(m, keep, (double*)F, sig, cx);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    qr_pos(ctx, dt, m, keep, F, al->data, cc->data);
    // C = R diag(sigma): scale column j by sigma_j  (scale_columns divides, so pass 1/sigma)
    scale_columns_kernel<<<64, 256, 0, ctx->stream>>>(keep, keep, (double*)cc->data, isig, cx);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    conj_transpose(ctx, dt, n, keep, E, n, ar->data, keep);  // AR = E^H
  } else {
    // W = sigma^-1 E^H M (keep x n) -> LQ: W = L Q; AR = Q, C = Sigma L; AL = E
    GB_CHECK_CUDA(cudaMemcpyAsync(al->data, E, (size_t)m * keep * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    gemm_fp64(ctx, dt, 'C', 'N', keep, n, m, cplx{1, 0}, E, m, 0, M, m, 0, cplx{0, 0}, F, keep, 0, 1);
    scale_rows_kernel<<<256, 256, 0, ctx->stream>>>(keep, n, (double*)F, keep, isig, cx);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    // LQ of W through the positive QR of W^H (n x keep)
    char* Wh = (char*)scratch(ctx, SLOT_T2, (size_t)n * keep * es + 256);
    conj_transpose(ctx, dt, keep, n, F, keep, Wh, n);
    char* Qp = (char*)scratch(ctx, SLOT_GAUGE2, (size_t)n * keep * es + 256);
    char* Rp = (char*)scratch(ctx, SLOT_RED, (size_t)keep * keep * es + 4096);
    qr_pos(ctx, dt, n, keep, Wh, Qp, Rp);
    conj_transpose(ctx, dt, n, keep, Qp, n, ar->data, keep);  // AR = Qp^H
    conj_transpose(ctx, dt, keep, keep, Rp, keep, cc->data, keep);  // L = Rp^H
    scale_rows_kernel<<<64, 256, 0, ctx->stream>>>(keep, keep, (double*)cc->data, keep, sig, cx);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
  }
  if (normalize) {
    double nc = nrm2(ctx, dt, keep * keep, cc->data);
    scale(ctx, dt, keep * keep, cplx{1.0 / nc, 0}, cc->data);
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *AL = al;
  *AR = ar;
  *S = cc;
  return true;
}

// env-transfer mix plans cached per (W, side, dims)
struct TransferKey {
  const gb_tensor* W;
  int side;
  int64_t a, b, c;
  bool operator<(const TransferKey& o) const {
    return std::tie(W, side, a, b, c) < std::tie(o.W, o.side, o.a, o.b, o.c);
  }
};
std::mutex g_tr_mu;
std::map<TransferKey, MixDev> g_tr_cache;

void drop_transfer_cache(const gb_tensor* W) {
  std::lock_guard<std::mutex> lk(g_tr_mu);
  for (auto it = g_tr_cache.begin(); it != g_tr_cache.end();) {
    if (it->first.W == W) {
      mix_free(it->second);
      it = g_tr_cache.erase(it);
    } else {
      ++it;
    }
  }
}

double wval(const gb_tensor* W, int64_t a, int64_t s, int64_t t, int64_t b, double* im) {
  int64_t i = a + W->dims[0] * (s + W->dims[1] * (t + W->dims[2] * b));
  if (is_cplx(W->dtype)) {
    *im = W->host_mpo[2 * i + 1];
    return W->host_mpo[2 * i];
  }
  *im = 0;
  return W->host_mpo[i];
}

const MixDev& transfer_plan(gb_ctx* ctx, const gb_tensor* W, int side, int64_t D1, int64_t D2,
                            int64_t D3, bool cx) {
  TransferKey key{W, side * 2 + (cx ? 1 : 0), D1, D2, D3};
  std::lock_guard<std::mutex> lk(g_tr_mu);
  auto it = g_tr_cache.find(key);
  if (it != g_tr_cache.end()) return it->second;
  const int64_t wl = W->dims[0], d = W->dims[1], wr = W->dims[3];
  MixPlan p;
  p.cplx = cx;
  if (side == 0) {
    // left: T1 (bra, s', kn, w) -> T2 (bra, s, kn, w'); D1 = Dbra, D2 = Dkn
    p.A = D1;
    p.N = D2;
    p.xa = 1;
    p.xn = D1 * d;
    p.ya = 1;
    p.yn = D1 * d;
    p.nI = d * wl;
    p.nJ = d * wr;
    p.in_off.resize(p.nI);
    p.out_off.resize(p.nJ);
    for (int64_t u = 0; u < d; ++u)
      for (int64_t w = 0; w < wl; ++w) p.in_off[u + d * w] = D1 * u + D1 * d * D2 * w;
    for (int64_t s = 0; s < d; ++s)
      for (int64_t v = 0; v < wr; ++v) p.out_off[s + d * v] = D1 * s + D1 * d * D2 * v;
    p.row_ptr.push_back(0);
    for (int64_t J = 0; J < p.nJ; ++J) {
      int64_t s = J % d, v = J / d;
      for (int64_t w = 0; w < wl; ++w)
        for (int64_t u = 0; u < d; ++u) {
          double im;
          double re = wval(W, w, s, u, v, &im);
          if (re == 0.0 && im == 0.0) continue;
          p.col.push_back((int)(u + d * w));
          p.val.push_back(re);
          if (cx) p.val.push_back(im);
        }
      p.row_ptr.push_back((int)p.col.size());
    }
  } else {
    // right: T1 (a, t, v, r) -> T2 (a, w, s, r); D1 = Dk, D3 = Dbra_r
    p.A = D1;
    p.N = D3;
    p.xa = 1;
    p.xn = D1 * d * wr;
    p.ya = 1;
    p.yn = D1 * wl * d;
    p.nI = d * wr;
    p.nJ = wl * d;
    p.in_off.resize(p.nI);
    p.out_off.resize(p.nJ);
    for (int64_t t = 0; t < d; ++t)
      for (int64_t v = 0; v < wr; ++v) p.in_off[t + d * v] = D1 * t + D1 * d * v;
    for (int64_t w = 0; w < wl; ++w)
      for (int64_t s = 0; s < d; ++s) p.out_off[w + wl * s] = D1 * w + D1 * wl * s;
    p.row_ptr.push_back(0);
    for (int64_t J = 0; J < p.nJ; ++J) {
      int64_t w = J % wl, s = J / wl;
      for (int64_t v = 0; v < wr; ++v)
        for (int64_t t = 0; t < d; ++t) {
          double im;
          double re = wval(W, w, s, t, v, &im);
          if (re == 0.0 && im == 0.0) continue;
          p.col.push_back((int)(t + d * v));
          p.val.push_back(re);
          if (cx) p.val.push_back(im);
        }
      p.row_ptr.push_back((int)p.col.size());
    }
  }
  MixDev m = mix_upload(ctx, p);
  auto res = g_tr_cache.emplace(key, m);
  return res.first->second;
}

void check_ctx(const gb_tensor* t, gb_ctx* ctx) {
  GB_REQUIRE(t, "null tensor");
  GB_REQUIRE(t->ctx == ctx, "tensor belongs to a different context");
}

}  // namespace

// external-linkage access to the gauge helpers above (used by u1.cu)
namespace gb {
gb_tensor* gauge_new_tensor(gb_ctx* ctx, int kind, int dtype, int ndim, const int64_t* dims) {
  return new_tensor(ctx, kind, dtype, ndim, dims);
}
void gauge_free_tensor(gb_tensor* t) { free_tensor(t); }
void gauge_qr_pos(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* M, void* Q, void* R) {
  qr_pos(ctx, dtype, m, n, M, Q, R);
}
void gauge_svd_tall(gb_ctx* ctx, int dtype, int64_t m, int64_t n, void* A, void* U, double* S,
                    void* VT) {
  svd_tall(ctx, dtype, m, n, A, U, S, VT);
}
void gauge_conj_transpose(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A,
                          int64_t lda, void* B, int64_t ldb) {
  conj_transpose(ctx, dtype, m, n, A, lda, B, ldb);
}
void* gauge_solver(gb_ctx* ctx) { return (void*)solver(ctx); }

// One host thread per lane, started with the first parallel call and kept until the context
// is destroyed (thread start-up stays off the per-call path).  A call hands every worker the
// same job and waits until all of them have finished it.
struct LanePool {
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  uint64_t gen = 0;
  int busy = 0;
  bool stop = false;
  std::function<void(int)> job;

  void start(int count, int device) {
    while ((int)threads.size() < count) {
      const int k = (int)threads.size();
      threads.emplace_back([this, k, device] {
        cudaSetDevice(device);
        uint64_t seen = 0;
        for (;;) {
          std::function<void(int)> f;
          {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || gen != seen; });
            if (stop) return;
            seen = gen;
            f = job;
          }
          f(k);
          {
            std::lock_guard<std::mutex> lk(mu);
            if (--busy == 0) cv_done.notify_all();
          }
        }
      });
    }
  }
  void run(const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> lk(mu);
      job = f;
      busy = (int)threads.size();
      ++gen;
    }
    cv_work.notify_all();
    std::unique_lock<std::mutex> lk(mu);
    cv_done.wait(lk, [&] { return busy == 0; });
  }
  ~LanePool() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    for (auto& t : threads) t.join();
  }
};

void run_on_lanes_at(gb_ctx* ctx, int64_t n, const char* file, int line,
                     const std::function<void(gb_ctx*, int64_t)>& fn) {
  const int K = (int)std::min<int64_t>(n, ctx->lane_max);
  if (K <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(ctx, i);
    return;
  }
  while ((int)ctx->lanes.size() < K) {
    gb_ctx* l = nullptr;
    const int rc = gb_ctx_create(ctx->device, 0, &l);
    if (rc != GB_OK) throw Error(rc, "lane context: " + std::string(gb_last_error()));
    l->lane = true;
    ctx->lanes.push_back(l);
  }
  std::vector<int64_t> before(K);
  for (int k = 0; k < K; ++k) {
    gb_ctx* l = ctx->lanes[k];
    l->svd_method = ctx->svd_method;
    l->eig_method = ctx->eig_method;
    l->aux_prec = ctx->aux_prec;
    l->gemm_schedule = ctx->gemm_schedule;
    l->gemm_bn = ctx->gemm_bn;
    l->wait_ns = ctx->wait_ns;
    before[k] = l->launches;
  }
  if (!ctx->lane_pool) ctx->lane_pool = new LanePool();
  ctx->lane_pool->start(K, ctx->device);
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  std::atomic<int64_t> next{0};
  std::exception_ptr err;
  std::mutex mu;
  ctx->lane_pool->run([&](int k) {
    if (k >= K) return;
    gb_ctx* l = ctx->lanes[k];
    try {
      for (int64_t i; (i = next++) < n;) {
        {
          std::lock_guard<std::mutex> g(mu);
          if (err) break;
        }
        fn(l, i);
      }
      GB_CHECK_CUDA(cudaStreamSynchronize(l->stream));
    } catch (...) {
      std::lock_guard<std::mutex> g(mu);
      if (!err) err = std::current_exception();
    }
  });
  // marks the end of the lanes' work on the (idle) main stream, charged to the caller
  if (ctx->tracing) trace_point(ctx, file, line);
  for (int k = 0; k < K; ++k) ctx->launches += ctx->lanes[k]->launches - before[k];
  if (err) std::rethrow_exception(err);
}
void u1_left_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* ql, const int32_t* qs,
                  const int32_t* qr, gb_tensor** AL, gb_tensor** C, int32_t* qk, int64_t* k);
void u1_right_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* ql, const int32_t* qs,
                   const int32_t* qr, gb_tensor** C, gb_tensor** AR, int32_t* qk, int64_t* k);
void u1_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, const int32_t* ql, const int32_t* qs1,
                  const int32_t* qs2, const int32_t* qr, int64_t maxdim, double atol,
                  int normalize, gb_tensor** AL, gb_tensor** S, gb_tensor** AR, int32_t* qk,
                  int64_t* k, double* eps);
}  // namespace gb

// ================================================================== C ABI
extern "C" {

int gb_version(void) { return 10000; }

const char* gb_last_error(void) { return g_last_error.c_str(); }

int gb_ctx_create(int device, uint32_t flags, gb_ctx** out) {
  API_BEGIN
  GB_REQUIRE(out, "null output");
  (void)flags;
  int n = 0;
  GB_CHECK_CUDA(cudaGetDeviceCount(&n));
  GB_REQUIRE(device >= 0 && device < n, "device index out of range");
  GB_CHECK_CUDA(cudaSetDevice(device));
  gb_ctx* c = new gb_ctx();
  c->device = device;
  GB_CHECK_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  GB_CHECK_CUDA(cudaMalloc(&c->d_status, 256));
  GB_CHECK_CUDA(cudaMemset(c->d_status, 0, 256));
  c->d_tile_counter = (unsigned int*)((char*)c->d_status + 128);
  c->d_work = (double*)((char*)c->d_status + 192);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  *out = c;
  API_END
}

int gb_ctx_destroy(gb_ctx* ctx) {
  API_BEGIN
  if (!ctx) return GB_OK;
  DevGuard g(ctx->device);
  delete ctx->lane_pool;  // joins the lane threads (idle between calls)
  ctx->lane_pool = nullptr;
  for (gb_ctx* l : ctx->lanes) gb_ctx_destroy(l);
  ctx->lanes.clear();
  cudaStreamSynchronize(ctx->stream);
  for (auto& s : ctx->scratch)
    if (s.ptr) cudaFree(s.ptr);
  if (ctx->solver) {
    cusolverDnDestroyParams((cusolverDnParams_t)ctx->solver_params);
    cusolverDnDestroy((cusolverDnHandle_t)ctx->solver);
  }
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  for (auto e : ctx->prof_events) cudaEventDestroy(e);
  for (auto e : ctx->trace_ev) cudaEventDestroy(e);
  if (ctx->trace_start) cudaEventDestroy(ctx->trace_start);
  for (auto e : ctx->prof_region)
    if (e) cudaEventDestroy(e);
  cudaFree(ctx->d_status);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  API_END
}

int gb_ctx_synchronize(gb_ctx* ctx) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END
}

int gb_ctx_kernel_launches(gb_ctx* ctx, int64_t* out) {
  API_BEGIN
  GB_REQUIRE(ctx && out, "null argument");
  *out = ctx->launches;
  API_END
}

int gb_ctx_device_status(gb_ctx* ctx, int32_t* out) {
  API_BEGIN
  GB_REQUIRE(ctx && out, "null argument");
  int32_t v = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&v, ctx->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
  GB_CHECK_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int32_t), ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = v;
  API_END
}

int gb_ctx_set_precision(gb_ctx* ctx, int precision) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(precision == GB_PREC_FP64 || precision == GB_PREC_BF16X3 ||
                 precision == GB_PREC_TF32X3,
             "unknown precision");
  ctx->aux_prec = precision;
  API_END
}

int gb_ctx_set_svd_method(gb_ctx* ctx, int method) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(method == GB_SVD_GESVD || method == GB_SVD_GESVDP || method == GB_SVD_GRAM,
             "unknown SVD method");
  ctx->svd_method = method;
  API_END
}

int gb_ctx_set_option(gb_ctx* ctx, int option, int64_t value) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  switch (option) {
    case GB_OPT_STAGED_MIX:
      GB_REQUIRE(value >= 0 && value <= 2, "staged_mix: 0, 1 or 2");
      ctx->staged_mix = (int)value;
      break;
    default: throw Error(GB_ERR_ARG, "unknown option");
  }
  API_END
}

int gb_ctx_set_gauge(gb_ctx* ctx, int eig_method, int lanes) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(eig_method == GB_EIG_SYEVD || eig_method == GB_EIG_SYEVJ ||
                 eig_method == GB_EIG_SYEVD_DEVICE,
             "unknown eigensolver");
  GB_REQUIRE(lanes >= 1 && lanes <= 32, "lanes must be in 1..32");
  ctx->eig_method = eig_method;
  ctx->lane_max = lanes;
  API_END
}

int gb_ctx_set_gemm_schedule(gb_ctx* ctx, int schedule, int tile_n) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(schedule == GB_SCHED_PERSISTENT || schedule == GB_SCHED_PERSISTENT_DENSE ||
                 schedule == GB_SCHED_TILE || schedule == GB_SCHED_GROUPED,
             "unknown GEMM schedule");
  GB_REQUIRE(tile_n == 0 || tile_n == 128 || tile_n == 256, "tile_n must be 0, 128 or 256");
  ctx->gemm_schedule = schedule;
  ctx->gemm_bn = tile_n;
  API_END
}

int gb_ctx_set_wait_bound(gb_ctx* ctx, double seconds) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(seconds >= 0.0 && seconds <= 60.0, "wait bound must lie in [0, 60] s");
  ctx->wait_ns = (unsigned long long)(seconds * 1e9);
  API_END
}

int gb_ctx_set_counting(gb_ctx* ctx, int on) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  ctx->counting = on != 0;
  API_END
}

int gb_ctx_read_work(gb_ctx* ctx, double* tile_flops, double* nonzero_flops, int reset) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  DevGuard g(ctx->device);
  double w[2] = {0.0, 0.0};
  GB_CHECK_CUDA(cudaMemcpyAsync(w, ctx->d_work, sizeof(w), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  if (tile_flops) *tile_flops = w[0];
  if (nonzero_flops) *nonzero_flops = w[1];
  if (reset) GB_CHECK_CUDA(cudaMemsetAsync(ctx->d_work, 0, sizeof(w), ctx->stream));
  API_END
}

int gb_ctx_trace_begin(gb_ctx* ctx) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  DevGuard g(ctx->device);
  if (!ctx->trace_start) GB_CHECK_CUDA(cudaEventCreate(&ctx->trace_start));
  ctx->trace_used = 0;
  ctx->tracing = true;
  GB_CHECK_CUDA(cudaEventRecord(ctx->trace_start, ctx->stream));
  API_END
}

int gb_ctx_trace_end(gb_ctx* ctx, int64_t* n_sites, double* total_ms) {
  API_BEGIN
  GB_REQUIRE(ctx && n_sites, "null argument");
  GB_REQUIRE(ctx->tracing, "trace_end without trace_begin");
  DevGuard g(ctx->device);
  ctx->tracing = false;
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  std::map<int, std::pair<double, int64_t>> acc;
  cudaEvent_t prev = ctx->trace_start;
  for (size_t i = 0; i < ctx->trace_used; ++i) {
    float ms = 0.f;
    GB_CHECK_CUDA(cudaEventElapsedTime(&ms, prev, ctx->trace_ev[i]));
    auto& a = acc[ctx->trace_site[i]];
    a.first += ms;
    a.second += 1;
    prev = ctx->trace_ev[i];
  }
  if (total_ms) {
    float ms = 0.f;
    if (ctx->trace_used) GB_CHECK_CUDA(cudaEventElapsedTime(&ms, ctx->trace_start, prev));
    *total_ms = ms;
  }
  ctx->trace_res_site.clear();
  ctx->trace_res_ms.clear();
  ctx->trace_res_n.clear();
  for (auto& kv : acc) {
    ctx->trace_res_site.push_back(kv.first);
    ctx->trace_res_ms.push_back(kv.second.first);
    ctx->trace_res_n.push_back(kv.second.second);
  }
  *n_sites = (int64_t)acc.size();
  API_END
}

int gb_ctx_trace_site(gb_ctx* ctx, int64_t i, char* name, size_t name_len, double* ms,
                      int64_t* events) {
  API_BEGIN
  GB_REQUIRE(ctx && name && name_len > 0 && ms && events, "null argument");
  GB_REQUIRE(i >= 0 && i < (int64_t)ctx->trace_res_site.size(), "trace_site: index out of range");
  std::string nm;
  {
    std::lock_guard<std::mutex> lk(g_site_mu);
    nm = g_site_names[ctx->trace_res_site[i]];
  }
  std::snprintf(name, name_len, "%s", nm.c_str());
  *ms = ctx->trace_res_ms[i];
  *events = ctx->trace_res_n[i];
  API_END
}

int gb_ctx_profile_begin(gb_ctx* ctx) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  DevGuard g(ctx->device);
  for (auto& e : ctx->prof_region)
    if (!e) GB_CHECK_CUDA(cudaEventCreate(&e));
  ctx->profiling = true;
  ctx->prof_used = 0;
  ctx->prof_flops = 0.0;
  ctx->prof_kind.clear();
  for (int k = 0; k < 2; ++k) ctx->prof_kind_flops[k] = 0.0;
  GB_CHECK_CUDA(cudaEventRecord(ctx->prof_region[0], ctx->stream));
  API_END
}

int gb_ctx_profile_end(gb_ctx* ctx, double* gemm_ms, int64_t* gemm_launches, double* gemm_flops,
                       double* region_ms) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(ctx->profiling, "profile_end without profile_begin");
  DevGuard g(ctx->device);
  GB_CHECK_CUDA(cudaEventRecord(ctx->prof_region[1], ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  double tot = 0.0;
  for (int k = 0; k < 2; ++k) {
    ctx->prof_res_ms[k] = 0.0;
    ctx->prof_res_n[k] = 0;
    ctx->prof_res_flops[k] = ctx->prof_kind_flops[k];
  }
  for (size_t i = 0; i + 1 < ctx->prof_used; i += 2) {
    float ms = 0.f;
    GB_CHECK_CUDA(cudaEventElapsedTime(&ms, ctx->prof_events[i], ctx->prof_events[i + 1]));
    tot += ms;
    const int k = (i / 2 < ctx->prof_kind.size()) ? ctx->prof_kind[i / 2] : 0;
    ctx->prof_res_ms[k] += ms;
    ctx->prof_res_n[k] += 1;
  }
  float rms = 0.f;
  GB_CHECK_CUDA(cudaEventElapsedTime(&rms, ctx->prof_region[0], ctx->prof_region[1]));
  if (gemm_ms) *gemm_ms = tot;
  if (gemm_launches) *gemm_launches = (int64_t)(ctx->prof_used / 2);
  if (gemm_flops) *gemm_flops = ctx->prof_flops;
  if (region_ms) *region_ms = rms;
  ctx->profiling = false;
  ctx->prof_used = 0;
  API_END
}

int gb_ctx_profile_kernel(gb_ctx* ctx, int kernel, double* ms, int64_t* launches,
                          double* flops) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  GB_REQUIRE(kernel == GB_PROF_PERSISTENT || kernel == GB_PROF_GROUPED, "unknown kernel family");
  if (ms) *ms = ctx->prof_res_ms[kernel];
  if (launches) *launches = ctx->prof_res_n[kernel];
  if (flops) *flops = ctx->prof_res_flops[kernel];
  API_END
}

int gb_tensor_create(gb_ctx* ctx, int kind, int dtype, int ndim, const int64_t* dims,
                     gb_tensor** out) {
  API_BEGIN
  GB_REQUIRE(out && dims, "null argument");
  DevGuard g(ctx->device);
  *out = new_tensor(ctx, kind, dtype, ndim, dims);
  API_END
}

int gb_tensor_pack(gb_ctx* ctx, const gb_tensor* t, gb_packed** out) {
  API_BEGIN
  GB_REQUIRE(ctx && out, "null argument");
  check_ctx(t, ctx);
  GB_REQUIRE(t->kind != GB_KIND_MPO, "pack: MPO tensors keep their host mirror; not packed");
  DevGuard g(ctx->device);
  *out = tensor_pack(ctx, t);
  API_END
}

int gb_packed_unpack(gb_ctx* ctx, const gb_packed* p, gb_tensor* out) {
  API_BEGIN
  GB_REQUIRE(ctx && p, "null argument");
  check_ctx(out, ctx);
  GB_REQUIRE(packed_ctx(p) == ctx, "packed tensor belongs to another context");
  DevGuard g(ctx->device);
  packed_unpack(ctx, p, out);
  API_END
}

int gb_packed_info(const gb_packed* p, int64_t* tiles_kept, int64_t* tiles_total,
                   size_t* bytes) {
  API_BEGIN
  GB_REQUIRE(p, "null argument");
  packed_info(p, tiles_kept, tiles_total, bytes);
  API_END
}

int gb_packed_free(gb_packed* p) {
  API_BEGIN
  if (!p) return GB_OK;
  DevGuard g(packed_ctx(p)->device);
  packed_free(p);
  API_END
}

int gb_tensor_free(gb_tensor* t) {
  API_BEGIN
  if (!t) return GB_OK;
  DevGuard g(t->ctx->device);
  if (t->kind == GB_KIND_MPO) drop_transfer_cache(t);
  free_tensor(t);
  API_END
}

int gb_tensor_shape(const gb_tensor* t, int* kind, int* dtype, int* ndim, int64_t* dims) {
  API_BEGIN
  GB_REQUIRE(t, "null tensor");
  if (kind) *kind = t->kind;
  if (dtype) *dtype = t->dtype;
  if (ndim) *ndim = t->ndim;
  if (dims)
    for (int i = 0; i < t->ndim; ++i) dims[i] = t->dims[i];
  API_END
}

int gb_tensor_upload(gb_tensor* t, const void* host, size_t bytes) {
  API_BEGIN
  GB_REQUIRE(t && (host || bytes == 0), "null argument");
  GB_REQUIRE(bytes == t->bytes, "upload: byte count does not match the tensor");
  gb_ctx* ctx = t->ctx;
  DevGuard g(ctx->device);
  if (t->kind == GB_KIND_MPO) memcpy(t->host_mpo.data(), host, bytes), drop_transfer_cache(t);
  if (bytes == 0) return GB_OK;
  if (!needs_permute(t->kind)) {
    GB_CHECK_CUDA(cudaMemcpyAsync(t->data, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  } else {
    void* tmp = scratch(ctx, SLOT_TMP, bytes);
    GB_CHECK_CUDA(cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    int64_t rs[6], ds[6];
    ref_strides(t->kind, t->ndim, t->dims, rs, ds);
    permute(ctx, t->dtype, t->ndim, t->dims, tmp, rs, t->data, ds);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  API_END
}

int gb_tensor_download(const gb_tensor* t, void* host, size_t bytes) {
  API_BEGIN
  GB_REQUIRE(t && (host || bytes == 0), "null argument");
  GB_REQUIRE(bytes == t->bytes, "download: byte count does not match the tensor");
  gb_ctx* ctx = t->ctx;
  DevGuard g(ctx->device);
  if (bytes == 0) return GB_OK;
  if (!needs_permute(t->kind)) {
    GB_CHECK_CUDA(cudaMemcpyAsync(host, t->data, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    void* tmp = scratch(ctx, SLOT_TMP, bytes);
    int64_t rs[6], ds[6];
    ref_strides(t->kind, t->ndim, t->dims, rs, ds);
    permute(ctx, t->dtype, t->ndim, t->dims, t->data, ds, tmp, rs);
    GB_CHECK_CUDA(cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END
}

int gb_tensor_copy(gb_tensor* dst, const gb_tensor* src) {
  API_BEGIN
  GB_REQUIRE(dst && src, "null tensor");
  GB_REQUIRE(dst->bytes == src->bytes && dst->dtype == src->dtype, "copy: size mismatch");
  GB_REQUIRE(dst->kind == src->kind || !needs_permute(dst->kind) == !needs_permute(src->kind),
             "copy: layout mismatch");
  DevGuard g(dst->ctx->device);
  GB_CHECK_CUDA(cudaMemcpyAsync(dst->data, src->data, src->bytes, cudaMemcpyDeviceToDevice,
                                dst->ctx->stream));
  API_END
}

// ---------------------------------------------------------------- Krylov basis helpers
// A basis is a GB_KIND_GENERIC tensor (n, kmax): column j holds a vector of n elements.  Used
// by host-driven Krylov loops over operators without a device solver of their own (the
// Arnoldi of the uniform gauge), so that one orthogonalisation is two passes of batched
// dot products and updates instead of one host round trip per basis vector.
static void basis_check(const gb_tensor* basis, const gb_tensor* v, int64_t j) {
  GB_REQUIRE(basis && v, "null tensor");
  GB_REQUIRE(basis->kind == GB_KIND_GENERIC && basis->ndim == 2, "basis: a 2-leg generic tensor");
  GB_REQUIRE(basis->dtype == v->dtype, "basis: dtypes");
  GB_REQUIRE(!needs_permute(v->kind), "basis: vectors in reference leg order only");
  GB_REQUIRE(numel(v) == basis->dims[0], "basis: vector length");
  GB_REQUIRE(j >= 0 && j <= basis->dims[1], "basis: column index");
}

int gb_basis_set(gb_ctx* ctx, gb_tensor* basis, int64_t j, const gb_tensor* v) {
  API_BEGIN
  check_ctx(basis, ctx);
  check_ctx(v, ctx);
  basis_check(basis, v, j);
  GB_REQUIRE(j < basis->dims[1], "basis: column index");
  DevGuard g(ctx->device);
  const size_t bytes = (size_t)basis->dims[0] * elem_size(v->dtype);
  GB_CHECK_CUDA(cudaMemcpyAsync((char*)basis->data + (size_t)j * bytes, v->data, bytes,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  API_END
}

int gb_basis_orthogonalize(gb_ctx* ctx, const gb_tensor* basis, int64_t k, gb_tensor* w,
                           double* h) {
  API_BEGIN
  check_ctx(basis, ctx);
  check_ctx(w, ctx);
  basis_check(basis, w, k);
  GB_REQUIRE(h || k == 0, "null output");
  DevGuard g(ctx->device);
  const int dt = w->dtype;
  const int64_t n = basis->dims[0];
  // classical Gram-Schmidt, two passes; h = the sum of both passes' projections
  std::vector<cplx> c1(k), c2(k), neg(k);
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<cplx>& c = pass ? c2 : c1;
    multi_dot(ctx, dt, n, (int)k, basis->data, n, w->data, c.data());
    for (int64_t j = 0; j < k; ++j) neg[j] = cplx{-c[j].re, -c[j].im};
    multi_axpy(ctx, dt, n, (int)k, basis->data, n, neg.data(), w->data);
  }
  for (int64_t j = 0; j < k; ++j) {
    h[2 * j] = c1[j].re + c2[j].re;
    h[2 * j + 1] = c1[j].im + c2[j].im;
  }
  API_END
}

int gb_basis_combine(gb_ctx* ctx, const gb_tensor* basis, int64_t k, const double* coef,
                     gb_tensor* out) {
  API_BEGIN
  check_ctx(basis, ctx);
  check_ctx(out, ctx);
  basis_check(basis, out, k);
  GB_REQUIRE(coef || k == 0, "null coefficients");
  DevGuard g(ctx->device);
  std::vector<cplx> c(k);
  const bool cx = is_cplx(out->dtype);
  for (int64_t j = 0; j < k; ++j) c[j] = cplx{coef[2 * j], cx ? coef[2 * j + 1] : 0.0};
  fill_zero(ctx, out->data, out->bytes);
  multi_axpy(ctx, out->dtype, basis->dims[0], (int)k, basis->data, basis->dims[0], c.data(),
             out->data);
  API_END
}

int gb_tensor_scale(gb_tensor* t, double re, double im) {
  API_BEGIN
  GB_REQUIRE(t, "null tensor");
  GB_REQUIRE(is_cplx(t->dtype) || im == 0.0, "scale: complex factor on a real tensor");
  DevGuard g(t->ctx->device);
  scale(t->ctx, t->dtype, numel(t), cplx{re, im}, t->data);
  API_END
}

int gb_tensor_axpy(gb_tensor* y, double re, double im, const gb_tensor* x) {
  API_BEGIN
  GB_REQUIRE(x && y, "null tensor");
  GB_REQUIRE(x->bytes == y->bytes && x->dtype == y->dtype, "axpy: size mismatch");
  GB_REQUIRE(is_cplx(y->dtype) || im == 0.0, "axpy: complex factor on a real tensor");
  DevGuard g(y->ctx->device);
  axpy(y->ctx, y->dtype, numel(y), cplx{re, im}, x->data, y->data);
  API_END
}

int gb_tensor_dot(const gb_tensor* x, const gb_tensor* y, double* re, double* im) {
  API_BEGIN
  GB_REQUIRE(x && y && re, "null argument");
  GB_REQUIRE(x->bytes == y->bytes && x->dtype == y->dtype, "dot: size mismatch");
  DevGuard g(x->ctx->device);
  cplx r = dot(x->ctx, x->dtype, numel(x), x->data, y->data);
  *re = r.re;
  if (im) *im = r.im;
  API_END
}

int gb_tensor_norm(const gb_tensor* x, double* out) {
  API_BEGIN
  GB_REQUIRE(x && out, "null argument");
  DevGuard g(x->ctx->device);
  *out = nrm2(x->ctx, x->dtype, numel(x), x->data);
  API_END
}

// ---------------------------------------------------------------- derivative operators
int gb_heff_build(gb_ctx* ctx, int kind, const gb_tensor* GL, const gb_tensor* W1,
                  const gb_tensor* W2, const gb_tensor* GR, int precision, gb_heff** out) {
  API_BEGIN
  GB_REQUIRE(ctx && out, "null argument");
  DevGuard g(ctx->device);
  if (GL) check_ctx(GL, ctx);
  if (GR) check_ctx(GR, ctx);
  *out = heff_build(ctx, kind, GL, W1, W2, GR, precision);
  API_END
}

int gb_heff_free(gb_heff* h) {
  API_BEGIN
  if (!h) return GB_OK;
  heff_free(h);
  API_END
}

int gb_heff_terms(const gb_heff* h, char* buf, size_t len) {
  API_BEGIN
  GB_REQUIRE(h && buf && len > 0, "null argument");
  HeffInfo hi = heff_info(h);
  snprintf(buf, len, "%s", hi.terms);
  API_END
}

int gb_heff_describe(const gb_heff* h, char* buf, size_t len) {
  API_BEGIN
  GB_REQUIRE(h && buf && len > 0, "null argument");
  snprintf(buf, len, "%s", heff_describe(h).c_str());
  API_END
}

int gb_heff_flops(const gb_heff* h, double* flops) {
  API_BEGIN
  GB_REQUIRE(h && flops, "null argument");
  *flops = heff_info(h).flops;
  API_END
}

int gb_heff_set_precision(gb_heff* h, int precision) {
  API_BEGIN
  GB_REQUIRE(h, "null operator");
  heff_set_precision(h, precision);
  API_END
}

int gb_heff_set_sectors(gb_heff* h, const int32_t* q_left, const int32_t* q_phys1,
                        const int32_t* q_phys2, const int32_t* q_right) {
  API_BEGIN
  GB_REQUIRE(h && q_left && q_phys1 && q_right, "null argument");
  HeffInfo hi = heff_info(h);
  GB_REQUIRE(hi.kind != GB_HEFF_C, "set_sectors: AC or AC2 operators only");
  GB_REQUIRE(hi.kind != GB_HEFF_AC2 || q_phys2, "set_sectors: AC2 needs both physical legs");
  DevGuard g(hi.ctx->device);
  heff_set_sectors(h, q_left, q_phys1, q_phys2, q_right);
  API_END
}

static void check_x(const gb_heff* h, const gb_tensor* x) {
  HeffInfo hi = heff_info(h);
  GB_REQUIRE(x, "null tensor");
  GB_REQUIRE(x->dtype == hi.dtype, "operator and vector dtypes differ");
  int want = hi.kind == GB_HEFF_AC2 ? GB_KIND_AC2 : (hi.kind == GB_HEFF_AC ? GB_KIND_MPS : GB_KIND_BOND);
  GB_REQUIRE(x->kind == want, "vector kind does not match the operator");
  for (int i = 0; i < hi.xndim; ++i) GB_REQUIRE(x->dims[i] == hi.xdims[i], "vector shape does not match the operator");
}

int gb_heff_apply(gb_heff* h, const gb_tensor* x, gb_tensor* y) {
  API_BEGIN
  GB_REQUIRE(h, "null operator");
  check_x(h, x);
  check_x(h, y);
  GB_REQUIRE(x != y, "apply: x and y must be distinct");
  HeffInfo hi = heff_info(h);
  DevGuard g(hi.ctx->device);
  heff_apply_raw(h, x->data, y->data);
  API_END
}

int gb_heff_eigsolve(gb_heff* h, gb_tensor* x, int krylovdim, int maxiter, double tol, int eager,
                     double* lambda, gb_krylov_info* info) {
  API_BEGIN
  GB_REQUIRE(h && lambda, "null argument");
  check_x(h, x);
  HeffInfo hi = heff_info(h);
  DevGuard g(hi.ctx->device);
  heff_eigsolve_raw(hi.ctx, h, hi.xnumel, hi.dtype, x->data, krylovdim, maxiter, tol, eager != 0,
                    lambda, info);
  API_END
}

int gb_heff_exponentiate(gb_heff* h, gb_tensor* x, double t_re, double t_im, int krylovdim,
                         int maxiter, double tol, gb_krylov_info* info) {
  API_BEGIN
  GB_REQUIRE(h, "null operator");
  check_x(h, x);
  HeffInfo hi = heff_info(h);
  DevGuard g(hi.ctx->device);
  heff_exponentiate_raw(hi.ctx, h, hi.xnumel, hi.dtype, x->data, t_re, t_im, krylovdim, maxiter,
                        tol, info);
  API_END
}

// ---------------------------------------------------------------- environments
int gb_env_transfer_left(gb_ctx* ctx, const gb_tensor* GL, const gb_tensor* W, const gb_tensor* A,
                         const gb_tensor* Abar, int precision, gb_tensor* GL_out) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  for (const gb_tensor* t : {GL, W, A, Abar, (const gb_tensor*)GL_out}) check_ctx(t, ctx);
  GB_REQUIRE(GL->kind == GB_KIND_GL && GL_out->kind == GB_KIND_GL, "transfer_left: GL kinds");
  GB_REQUIRE(W->kind == GB_KIND_MPO && A->kind == GB_KIND_MPS && Abar->kind == GB_KIND_MPS,
             "transfer_left: operand kinds");
  const int dt = GL->dtype;
  GB_REQUIRE(A->dtype == dt && Abar->dtype == dt && GL_out->dtype == dt, "transfer_left: dtypes");
  GB_REQUIRE(!(is_cplx(W->dtype) && !is_cplx(dt)), "transfer_left: complex MPO on real env");
  const int64_t Dbra = GL->dims[0], wl = GL->dims[1], Dket = GL->dims[2];
  const int64_t d = W->dims[1], wr = W->dims[3];
  GB_REQUIRE(W->dims[0] == wl && W->dims[2] == d, "transfer_left: MPO shape");
  GB_REQUIRE(A->dims[0] == Dket && A->dims[1] == d, "transfer_left: ket tensor shape");
  GB_REQUIRE(Abar->dims[0] == Dbra && Abar->dims[1] == d, "transfer_left: bra tensor shape");
  const int64_t Dkn = A->dims[2], Dbn = Abar->dims[2];
  GB_REQUIRE(GL_out->dims[0] == Dbn && GL_out->dims[1] == wr && GL_out->dims[2] == Dkn,
             "transfer_left: output shape");
  DevGuard g(ctx->device);
  const size_t es = elem_size(dt);
  int prec = precision;
  void* T1 = scratch(ctx, SLOT_T1, (size_t)Dbra * d * Dkn * wl * es);
  void* T2 = scratch(ctx, SLOT_T2, (size_t)Dbra * d * Dkn * wr * es);
  // T1[bra, (s' kn), w] = GL[bra, ket, w] A[ket, (s' kn)]  (batched over w)
  gemm(ctx, prec, dt, 'N', 'N', Dbra, d * Dkn, Dket, 1.0, GL->data, Dbra, Dbra * Dket, A->data,
       Dket, 0, 0.0, T1, Dbra, Dbra * d * Dkn, wl);
  // T2[bra, s, kn, w'] = W[w, s, s', w'] T1[bra, s', kn, w]
  const MixDev& m = transfer_plan(ctx, W, 0, Dbra, Dkn, 0, is_cplx(dt));
  mix_run(ctx, m, dt, T1, T2, 0.0);
  // GL'[bn, (kn w')] = conj(Abar)[(bra s), bn]^T T2[(bra s), (kn w')]
  gemm(ctx, prec, dt, 'C', 'N', Dbn, Dkn * wr, Dbra * d, 1.0, Abar->data, Dbra * d, 0, T2,
       Dbra * d, 0, 0.0, GL_out->data, Dbn, 0);
  API_END
}

int gb_env_transfer_right(gb_ctx* ctx, const gb_tensor* GR, const gb_tensor* W, const gb_tensor* A,
                          const gb_tensor* Abar, int precision, gb_tensor* GR_out) {
  API_BEGIN
  GB_REQUIRE(ctx, "null context");
  for (const gb_tensor* t : {GR, W, A, Abar, (const gb_tensor*)GR_out}) check_ctx(t, ctx);
  GB_REQUIRE(GR->kind == GB_KIND_GR && GR_out->kind == GB_KIND_GR, "transfer_right: GR kinds");
  GB_REQUIRE(W->kind == GB_KIND_MPO && A->kind == GB_KIND_MPS && Abar->kind == GB_KIND_MPS,
             "transfer_right: operand kinds");
  const int dt = GR->dtype;
  GB_REQUIRE(A->dtype == dt && Abar->dtype == dt && GR_out->dtype == dt, "transfer_right: dtypes");
  GB_REQUIRE(!(is_cplx(W->dtype) && !is_cplx(dt)), "transfer_right: complex MPO on real env");
  const int64_t Dket = GR->dims[0], wr = GR->dims[1], Dbra = GR->dims[2];
  const int64_t wl = W->dims[0], d = W->dims[1];
  GB_REQUIRE(W->dims[3] == wr && W->dims[2] == d, "transfer_right: MPO shape");
  GB_REQUIRE(A->dims[2] == Dket && A->dims[1] == d, "transfer_right: ket tensor shape");
  GB_REQUIRE(Abar->dims[2] == Dbra && Abar->dims[1] == d, "transfer_right: bra tensor shape");
  const int64_t Dk = A->dims[0], Db = Abar->dims[0];
  GB_REQUIRE(GR_out->dims[0] == Dk && GR_out->dims[1] == wl && GR_out->dims[2] == Db,
             "transfer_right: output shape");
  DevGuard g(ctx->device);
  const size_t es = elem_size(dt);
  int prec = precision;
  void* T1 = scratch(ctx, SLOT_T1, (size_t)Dk * d * wr * Dbra * es);
  void* T2 = scratch(ctx, SLOT_T2, (size_t)Dk * wl * d * Dbra * es);
  // T1[(a t), (v r)] = A[(a t), q] GR[q, (v r)]
  gemm(ctx, prec, dt, 'N', 'N', Dk * d, wr * Dbra, Dket, 1.0, A->data, Dk * d, 0, GR->data, Dket,
       0, 0.0, T1, Dk * d, 0);
  // T2[a, w, s, r] = W[w, s, t, v] T1[a, t, v, r]
  const MixDev& m = transfer_plan(ctx, W, 1, Dk, 0, Dbra, is_cplx(dt));
  mix_run(ctx, m, dt, T1, T2, 0.0);
  // GR'[(a w), b] = T2[(a w), (s r)] conj(Abar[b, (s r)])^T
  gemm(ctx, prec, dt, 'N', 'C', Dk * wl, Db, d * Dbra, 1.0, T2, Dk * wl, 0, Abar->data, Db, 0, 0.0,
       GR_out->data, Dk * wl, 0);
  API_END
}

// ---------------------------------------------------------------- projections
int gb_mpo_project(gb_ctx* ctx, const gb_tensor* GL, const gb_tensor* W, const gb_tensor* GR,
                   const gb_tensor* x, int precision, gb_tensor* y) {
  API_BEGIN
  GB_REQUIRE(ctx && GL && GR && x && y, "null argument");
  for (const gb_tensor* t : {GL, GR, x, (const gb_tensor*)y}) check_ctx(t, ctx);
  if (W) check_ctx(W, ctx);
  GB_REQUIRE(GL->kind == GB_KIND_GL && GR->kind == GB_KIND_GR, "project: environment kinds");
  const int dt = x->dtype;
  GB_REQUIRE(GL->dtype == dt && GR->dtype == dt && y->dtype == dt, "project: dtypes");
  // GL[bra l, w, ket l'] (device (a, a', w)); GR[ket r', w, bra r] (device (b', w, b))
  const int64_t Dlb = GL->dims[0], wl = GL->dims[1], Dlk = GL->dims[2];
  const int64_t Drk = GR->dims[0], wr = GR->dims[1], Drb = GR->dims[2];
  DevGuard g(ctx->device);
  const size_t es = elem_size(dt);
  if (!W) {
    // C_projection: y[l, r] = GL[l w; l'] x[l'; r'] GR[r' w; r]
    GB_REQUIRE(x->kind == GB_KIND_BOND && y->kind == GB_KIND_BOND, "project: bond tensors");
    GB_REQUIRE(wl == wr, "project: environment channels differ");
    GB_REQUIRE(x->dims[0] == Dlk && x->dims[1] == Drk, "project: x shape (ket bonds)");
    GB_REQUIRE(y->dims[0] == Dlb && y->dims[1] == Drb, "project: y shape (bra bonds)");
    void* T1 = scratch(ctx, SLOT_T1, (size_t)Dlk * wr * Drb * es);
    // T1[l', (w r)] = x[l', r'] GR[r', (w r)];  y[l, r] = GL[l, (l' w)] T1[(l' w), r]
    gemm(ctx, precision, dt, 'N', 'N', Dlk, wr * Drb, Drk, 1.0, x->data, Dlk, 0, GR->data, Drk,
         0, 0.0, T1, Dlk, 0);
    gemm(ctx, precision, dt, 'N', 'N', Dlb, Drb, Dlk * wl, 1.0, GL->data, Dlb, 0, T1, Dlk * wl,
         0, 0.0, y->data, Dlb, 0);
  } else {
    // AC_projection: y[l s; r] = GL[l w; l'] x[l' s'; r'] W[w s; s' w'] GR[r' w'; r]
    GB_REQUIRE(W->kind == GB_KIND_MPO, "project: W must be an MPO tensor");
    GB_REQUIRE(!(is_cplx(W->dtype) && !is_cplx(dt)), "project: complex MPO on real data");
    GB_REQUIRE(x->kind == GB_KIND_MPS && y->kind == GB_KIND_MPS, "project: MPS tensors");
    const int64_t d = W->dims[1];
    GB_REQUIRE(W->dims[0] == wl && W->dims[3] == wr && W->dims[2] == d, "project: MPO shape");
    GB_REQUIRE(x->dims[0] == Dlk && x->dims[1] == d && x->dims[2] == Drk,
               "project: x shape (ket bonds)");
    GB_REQUIRE(y->dims[0] == Dlb && y->dims[1] == d && y->dims[2] == Drb,
               "project: y shape (bra bonds)");
    void* T1 = scratch(ctx, SLOT_T1, (size_t)Dlk * d * wr * Drb * es);
    void* T2 = scratch(ctx, SLOT_T2, (size_t)Dlk * wl * d * Drb * es);
    // T1[(l' s'), (w' r)] = x[(l' s'), r'] GR[r', (w' r)]  (the first step of transfer_right)
    gemm(ctx, precision, dt, 'N', 'N', Dlk * d, wr * Drb, Drk, 1.0, x->data, Dlk * d, 0,
         GR->data, Drk, 0, 0.0, T1, Dlk * d, 0);
    // T2[l', w, s, r] = W[w, s, s', w'] T1[l', s', w', r]
    const MixDev& m = transfer_plan(ctx, W, 1, Dlk, 0, Drb, is_cplx(dt));
    mix_run(ctx, m, dt, T1, T2, 0.0);
    // y[l, (s r)] = GL[l, (l' w)] T2[(l' w), (s r)]
    gemm(ctx, precision, dt, 'N', 'N', Dlb, d * Drb, Dlk * wl, 1.0, GL->data, Dlb, 0, T2,
         Dlk * wl, 0, 0.0, y->data, Dlb, 0);
  }
  API_END
}

// ---------------------------------------------------------------- bond expansion
int gb_mps_perturb(gb_ctx* ctx, int side, const gb_tensor* env, const gb_tensor* W,
                   const gb_tensor* AC, int precision, gb_tensor* out) {
  API_BEGIN
  GB_REQUIRE(ctx && env && W && AC && out, "null argument");
  for (const gb_tensor* t : {env, W, AC, (const gb_tensor*)out}) check_ctx(t, ctx);
  GB_REQUIRE(side == 0 || side == 1, "perturb: side must be 0 (left env) or 1 (right env)");
  GB_REQUIRE(W->kind == GB_KIND_MPO && AC->kind == GB_KIND_MPS && out->kind == GB_KIND_MPS,
             "perturb: operand kinds");
  const int dt = AC->dtype;
  GB_REQUIRE(env->dtype == dt && out->dtype == dt, "perturb: dtypes");
  GB_REQUIRE(!(is_cplx(W->dtype) && !is_cplx(dt)), "perturb: complex MPO on a real state");
  const int64_t Dl = AC->dims[0], d = AC->dims[1], Dr = AC->dims[2];
  const int64_t wl = W->dims[0], wr = W->dims[3];
  GB_REQUIRE(W->dims[1] == d && W->dims[2] == d, "perturb: MPO physical legs");
  DevGuard g(ctx->device);
  const size_t es = elem_size(dt);
  if (side == 0) {
    // P[l, s, (r w')] = GL[l, l', w] AC[l', s', r] W[w, s, s', w']  -- the first two steps
    // of transfer_left with the bra contraction left out
    GB_REQUIRE(env->kind == GB_KIND_GL && env->dims[1] == wl && env->dims[2] == Dl,
               "perturb: GL shape");
    const int64_t Db = env->dims[0];
    GB_REQUIRE(out->dims[0] == Db && out->dims[1] == d && out->dims[2] == Dr * wr,
               "perturb: output shape (Dl, d, Dr * wr)");
    void* T1 = scratch(ctx, SLOT_T1, (size_t)Db * d * Dr * wl * es);
    gemm(ctx, precision, dt, 'N', 'N', Db, d * Dr, Dl, 1.0, env->data, Db, Db * Dl, AC->data,
         Dl, 0, 0.0, T1, Db, Db * d * Dr, wl);
    const MixDev& m = transfer_plan(ctx, W, 0, Db, Dr, 0, is_cplx(dt));
    mix_run(ctx, m, dt, T1, out->data, 0.0);
  } else {
    // P[(l w), s, r] = W[w, s, s', w'] AC[l, s', r'] GR[r', w', r]  -- the first two steps of
    // transfer_right without the bra
    GB_REQUIRE(env->kind == GB_KIND_GR && env->dims[0] == Dr && env->dims[1] == wr,
               "perturb: GR shape");
    const int64_t Db = env->dims[2];
    GB_REQUIRE(out->dims[0] == Dl * wl && out->dims[1] == d && out->dims[2] == Db,
               "perturb: output shape (Dl * wl, d, Dr)");
    void* T1 = scratch(ctx, SLOT_T1, (size_t)Dl * d * wr * Db * es);
    gemm(ctx, precision, dt, 'N', 'N', Dl * d, wr * Db, Dr, 1.0, AC->data, Dl * d, 0, env->data,
         Dr, 0, 0.0, T1, Dl * d, 0);
    const MixDev& m = transfer_plan(ctx, W, 1, Dl, 0, Db, is_cplx(dt));
    mix_run(ctx, m, dt, T1, out->data, 0.0);
  }
  API_END
}

int gb_mps_cat(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* B, int leg, gb_tensor* out) {
  API_BEGIN
  GB_REQUIRE(ctx && A && out, "null argument");
  check_ctx(A, ctx);
  check_ctx(out, ctx);
  if (B) check_ctx(B, ctx);
  GB_REQUIRE(A->kind == GB_KIND_MPS && out->kind == GB_KIND_MPS && (!B || B->kind == GB_KIND_MPS),
             "cat: MPS tensors only");
  GB_REQUIRE(leg == 0 || leg == 2, "cat: leg must be 0 (left bond) or 2 (right bond)");
  GB_REQUIRE(out->dtype == A->dtype && (!B || B->dtype == A->dtype), "cat: dtypes");
  const int other = 2 - leg;
  GB_REQUIRE(out->dims[1] == A->dims[1] && out->dims[other] == A->dims[other],
             "cat: the legs not concatenated must agree");
  const int64_t nb = out->dims[leg] - A->dims[leg];
  GB_REQUIRE(nb >= 0, "cat: output smaller than the first operand");
  if (B)
    GB_REQUIRE(B->dims[1] == A->dims[1] && B->dims[other] == A->dims[other] && B->dims[leg] == nb,
               "cat: second operand shape");
  DevGuard g(ctx->device);
  const size_t es = elem_size(A->dtype);
  cudaStream_t st = ctx->stream;
  if (!B) GB_CHECK_CUDA(cudaMemsetAsync(out->data, 0, out->bytes, st));
  if (leg == 2) {  // right bond: slowest in (l, s, r) -- two contiguous pieces
    if (A->bytes)
      GB_CHECK_CUDA(cudaMemcpyAsync(out->data, A->data, A->bytes, cudaMemcpyDeviceToDevice, st));
    if (B && B->bytes)
      GB_CHECK_CUDA(cudaMemcpyAsync((char*)out->data + A->bytes, B->data, B->bytes,
                                    cudaMemcpyDeviceToDevice, st));
  } else {  // left bond: fastest -- row blocks of A->dims[0] and nb elements per (s, r)
    const int64_t cols = A->dims[1] * A->dims[2], ld = out->dims[0];
    if (A->dims[0] && cols)
      GB_CHECK_CUDA(cudaMemcpy2DAsync(out->data, ld * es, A->data, A->dims[0] * es,
                                      A->dims[0] * es, cols, cudaMemcpyDeviceToDevice, st));
    if (B && nb && cols)
      GB_CHECK_CUDA(cudaMemcpy2DAsync((char*)out->data + A->dims[0] * es, ld * es, B->data,
                                      nb * es, nb * es, cols, cudaMemcpyDeviceToDevice, st));
  }
  API_END
}

// out(i, s, r) = A(perm[i], s, r) (leg 0) or out(l, s, i) = A(l, s, perm[i]) (leg 2); element
// words of 8 bytes (a complex element is two)
__global__ void leg_permute_kernel(int64_t n0, int64_t mid, int64_t n2, int leg, int words,
                                   const int64_t* __restrict__ perm,
                                   const double* __restrict__ A, double* __restrict__ out) {
  const int64_t total = n0 * mid * n2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n0, rest = e / n0, s = rest % mid, r = rest / mid;
    const int64_t src = leg == 0 ? perm[i] + n0 * (s + mid * r) : i + n0 * (s + mid * perm[r]);
    for (int w = 0; w < words; ++w) out[words * e + w] = A[words * src + w];
  }
}

int gb_mps_permute(gb_ctx* ctx, const gb_tensor* A, int leg, const int64_t* perm,
                   gb_tensor* out) {
  API_BEGIN
  GB_REQUIRE(ctx && A && out && perm, "null argument");
  check_ctx(A, ctx);
  check_ctx(out, ctx);
  GB_REQUIRE(A->kind == GB_KIND_MPS && out->kind == GB_KIND_MPS, "permute: MPS tensors only");
  GB_REQUIRE(leg == 0 || leg == 2, "permute: leg must be 0 (left bond) or 2 (right bond)");
  GB_REQUIRE(out->dtype == A->dtype && out->dims[0] == A->dims[0] &&
                 out->dims[1] == A->dims[1] && out->dims[2] == A->dims[2],
             "permute: output shape");
  const int64_t n = A->dims[leg];
  std::vector<char> seen(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    GB_REQUIRE(perm[i] >= 0 && perm[i] < n && !seen[perm[i]], "permute: not a permutation");
    seen[perm[i]] = 1;
  }
  DevGuard g(ctx->device);
  int64_t* dp = (int64_t*)scratch(ctx, SLOT_TMP2, (size_t)std::max<int64_t>(n, 1) * 8 + 256);
  GB_CHECK_CUDA(cudaMemcpyAsync(dp, perm, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream));
  const int64_t total = numel(A);
  if (total) {
    const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096));
    leg_permute_kernel<<<nb, 256, 0, ctx->stream>>>(
        A->dims[0], A->dims[1], A->dims[2], leg, is_cplx(A->dtype) ? 2 : 1, dp,
        (const double*)A->data, (double*)out->data);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // perm is borrowed for the call only
  API_END
}

int gb_tensor_reshape(gb_tensor* t, int kind, int ndim, const int64_t* dims) {
  API_BEGIN
  GB_REQUIRE(t && dims, "null argument");
  auto plain = [](int k) {
    return k == GB_KIND_MPS || k == GB_KIND_AC2 || k == GB_KIND_BOND || k == GB_KIND_GENERIC;
  };
  GB_REQUIRE(plain(t->kind) && plain(kind), "reshape: MPS, two-site, bond or generic tensors");
  const int want = kind == GB_KIND_MPS ? 3 : kind == GB_KIND_AC2 ? 4 : kind == GB_KIND_BOND ? 2 : -1;
  GB_REQUIRE(ndim >= 1 && ndim <= 6 && (want < 0 || ndim == want), "reshape: rank");
  int64_t n = 1;
  for (int i = 0; i < ndim; ++i) {
    GB_REQUIRE(dims[i] >= 0, "reshape: negative dimension");
    n *= dims[i];
  }
  GB_REQUIRE(n == numel(t), "reshape: element count");
  t->kind = kind;
  t->ndim = ndim;
  for (int i = 0; i < 6; ++i) t->dims[i] = i < ndim ? dims[i] : 0;
  API_END
}

int gb_project_complement_right(gb_ctx* ctx, gb_tensor* Y, const gb_tensor* X) {
  API_BEGIN
  check_ctx(Y, ctx);
  check_ctx(X, ctx);
  GB_REQUIRE(X->kind == GB_KIND_MPS, "project_complement_right: X must be an MPS tensor");
  GB_REQUIRE(Y->kind == GB_KIND_MPS || Y->kind == GB_KIND_AC2,
             "project_complement_right: Y kind");
  GB_REQUIRE(X->dtype == Y->dtype, "project_complement_right: dtypes");
  const int64_t k = X->dims[0], cols = X->dims[1] * X->dims[2];
  GB_REQUIRE(cols > 0 && numel(Y) % cols == 0, "project_complement_right: trailing legs mismatch");
  // the trailing legs of Y in device order must be X's (s, r)
  if (Y->kind == GB_KIND_AC2)
    GB_REQUIRE(Y->dims[3] == X->dims[1] && Y->dims[2] == X->dims[2],
               "project_complement_right: trailing legs mismatch");
  else
    GB_REQUIRE(Y->dims[1] == X->dims[1] && Y->dims[2] == X->dims[2],
               "project_complement_right: trailing legs mismatch");
  const int64_t rows = numel(Y) / cols;
  DevGuard g(ctx->device);
  const size_t es = elem_size(Y->dtype);
  void* T = scratch(ctx, SLOT_TMP, (size_t)rows * k * es);
  // T = Y X^H (rows x k); Y -= T X
  gemm(ctx, ctx->aux_prec, Y->dtype, 'N', 'C', rows, k, cols, 1.0, Y->data, rows, 0, X->data, k,
       0, 0.0, T, rows, 0);
  gemm(ctx, ctx->aux_prec, Y->dtype, 'N', 'N', rows, cols, k, -1.0, T, rows, 0, X->data, k, 0,
       1.0, Y->data, rows, 0);
  API_END
}

int gb_env_linsolve(gb_ctx* ctx, int side, const gb_tensor* W, const gb_tensor* A, int precision,
                    const gb_tensor* lvec, const gb_tensor* rvec, const gb_tensor* b,
                    gb_tensor* x, int krylovdim, int maxiter, double tol, gb_krylov_info* info) {
  API_BEGIN
  check_ctx(b, ctx);
  check_ctx(x, ctx);
  GB_REQUIRE(W && A, "null argument");
  GB_REQUIRE(side == 0 || side == 1, "linsolve: side must be 0 (left) or 1 (right)");
  GB_REQUIRE(b->kind == (side == 0 ? GB_KIND_GL : GB_KIND_GR) && x->kind == b->kind,
             "linsolve: b and x must be environments of the side");
  GB_REQUIRE(b->dtype == x->dtype && b->ndim == 3 && x->ndim == 3 &&
                 std::equal(b->dims, b->dims + 3, x->dims),
             "linsolve: b and x must have the same shape");
  GB_REQUIRE((lvec == nullptr) == (rvec == nullptr), "linsolve: give both lvec and rvec or none");
  GB_REQUIRE(precision == GB_PREC_FP64 || precision == GB_PREC_BF16X3 ||
                 precision == GB_PREC_TF32X3,
             "linsolve: precision");
  DevGuard g(ctx->device);
  gb::env_linsolve_raw(ctx, side, W, A, precision, lvec, rvec, b, x, krylovdim, maxiter, tol,
                       info);
  API_END
}

int gb_env_regularize(gb_ctx* ctx, gb_tensor* env, int64_t chan, const gb_tensor* lvec,
                      const gb_tensor* rvec) {
  API_BEGIN
  GB_REQUIRE(ctx && env && lvec && rvec, "null argument");
  GB_REQUIRE(env->kind == GB_KIND_GL || env->kind == GB_KIND_GR, "regularize: env kind");
  GB_REQUIRE(lvec->kind == GB_KIND_BOND && rvec->kind == GB_KIND_BOND, "regularize: vec kinds");
  DevGuard g(ctx->device);
  const int dt = env->dtype;
  const int64_t D0 = env->dims[0], w = env->dims[1], D2 = env->dims[2];
  GB_REQUIRE(chan >= 0 && chan < w, "regularize: channel out of range");
  GB_REQUIRE(lvec->dims[0] == D2 && lvec->dims[1] == D0, "regularize: lvec shape");
  GB_REQUIRE(rvec->dims[0] == D0 && rvec->dims[1] == D2, "regularize: rvec shape");
  // v = channel slice as a D0 x D2 matrix; lambda = tr(lvec v) = sum lvec[j, i] v[i, j]
  const size_t es = elem_size(dt);
  void* vt = scratch(ctx, SLOT_TMP, (size_t)D0 * D2 * es);
  int64_t dims[2] = {D0, D2};
  int64_t ins[2], outs[2] = {1, D0};
  if (env->kind == GB_KIND_GL) {  // dev (a, a', w): slice contiguous
    ins[0] = 1;
    ins[1] = D0;
  } else {  // dev (b', w, b)
    ins[0] = 1;
    ins[1] = D0 * w;
  }
  const char* base = (const char*)env->data +
                     (size_t)(env->kind == GB_KIND_GL ? D0 * D2 * chan : D0 * chan) * es;
  permute(ctx, dt, 2, dims, base, ins, vt, outs);
  // tr(lvec v) = sum_{i,j} lvec[j, i] v[i, j] = <conj(lvec^T), v>
  void* lt = scratch(ctx, SLOT_TMP2, (size_t)D0 * D2 * es);
  conj_transpose(ctx, dt, D2, D0, lvec->data, D2, lt, D0);  // lt = lvec^H (D0 x D2)
  cplx lam = dot(ctx, dt, D0 * D2, lt, vt);                 // sum conj(lt) v = sum lvec^T v
  // v -= lam * rvec, written back into the slice
  axpy(ctx, dt, D0 * D2, cplx{-lam.re, -lam.im}, rvec->data, vt);
  permute(ctx, dt, 2, dims, vt, outs, (void*)base, ins);
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END
}

int gb_env_channel_copy(gb_ctx* ctx, gb_tensor* dst, int64_t dst_c0, const gb_tensor* src,
                        int64_t src_c0, int64_t nchan) {
  API_BEGIN
  check_ctx(dst, ctx);
  check_ctx(src, ctx);
  GB_REQUIRE(dst->kind == src->kind && (dst->kind == GB_KIND_GL || dst->kind == GB_KIND_GR),
             "channel_copy: both tensors must be environments of the same kind");
  GB_REQUIRE(dst->dtype == src->dtype, "channel_copy: dtypes");
  GB_REQUIRE(dst->dims[0] == src->dims[0] && dst->dims[2] == src->dims[2],
             "channel_copy: bond dimensions differ");
  GB_REQUIRE(nchan >= 0 && src_c0 >= 0 && dst_c0 >= 0 && src_c0 + nchan <= src->dims[1] &&
                 dst_c0 + nchan <= dst->dims[1],
             "channel_copy: channel range out of bounds");
  if (nchan == 0) return GB_OK;
  DevGuard g(ctx->device);
  const size_t es = elem_size(dst->dtype);
  const int64_t D0 = dst->dims[0], D2 = dst->dims[2];
  if (dst->kind == GB_KIND_GL) {  // device (a, a', w): a channel slice is contiguous
    GB_CHECK_CUDA(cudaMemcpyAsync((char*)dst->data + (size_t)D0 * D2 * dst_c0 * es,
                                  (const char*)src->data + (size_t)D0 * D2 * src_c0 * es,
                                  (size_t)D0 * D2 * nchan * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
  } else {  // device (b', w, b): D0*nchan contiguous elements per b
    GB_CHECK_CUDA(cudaMemcpy2DAsync((char*)dst->data + (size_t)D0 * dst_c0 * es,
                                    (size_t)D0 * dst->dims[1] * es,
                                    (const char*)src->data + (size_t)D0 * src_c0 * es,
                                    (size_t)D0 * src->dims[1] * es, (size_t)D0 * nchan * es, D2,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
  }
  API_END
}

int gb_tensor_adjoint(gb_ctx* ctx, const gb_tensor* C, gb_tensor* out) {
  API_BEGIN
  check_ctx(C, ctx);
  check_ctx(out, ctx);
  GB_REQUIRE(C->kind == GB_KIND_BOND && out->kind == GB_KIND_BOND, "adjoint: bond tensors only");
  GB_REQUIRE(C->dtype == out->dtype, "adjoint: dtypes");
  GB_REQUIRE(out->dims[0] == C->dims[1] && out->dims[1] == C->dims[0], "adjoint: output shape");
  DevGuard g(ctx->device);
  conj_transpose(ctx, C->dtype, C->dims[0], C->dims[1], C->data, C->dims[0], out->data,
                 C->dims[1]);
  API_END
}

// ---------------------------------------------------------------- state manipulation
int gb_mps_ac2(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* B, gb_tensor* AC2) {
  API_BEGIN
  for (const gb_tensor* t : {A, B, (const gb_tensor*)AC2}) check_ctx(t, ctx);
  GB_REQUIRE(A->kind == GB_KIND_MPS && B->kind == GB_KIND_MPS && AC2->kind == GB_KIND_AC2,
             "mps_ac2: kinds");
  GB_REQUIRE(A->dtype == B->dtype && A->dtype == AC2->dtype, "mps_ac2: dtypes");
  const int64_t Dl = A->dims[0], d1 = A->dims[1], m = A->dims[2];
  const int64_t d2 = B->dims[1], Dr = B->dims[2];
  GB_REQUIRE(B->dims[0] == m, "mps_ac2: bond mismatch");
  GB_REQUIRE(AC2->dims[0] == Dl && AC2->dims[1] == d1 && AC2->dims[2] == Dr && AC2->dims[3] == d2,
             "mps_ac2: output shape");
  DevGuard g(ctx->device);
  gemm(ctx, ctx->aux_prec, A->dtype, 'N', 'N', Dl * d1, d2 * Dr, m, 1.0, A->data, Dl * d1, 0,
       B->data, m, 0, 0.0, AC2->data, Dl * d1, 0);
  API_END
}

int gb_mps_mul_front(gb_ctx* ctx, const gb_tensor* C, const gb_tensor* A, gb_tensor* out) {
  API_BEGIN
  for (const gb_tensor* t : {C, A, (const gb_tensor*)out}) check_ctx(t, ctx);
  GB_REQUIRE(C->kind == GB_KIND_BOND && A->kind == GB_KIND_MPS && out->kind == GB_KIND_MPS,
             "mul_front: kinds");
  GB_REQUIRE(C->dtype == A->dtype && out->dtype == A->dtype, "mul_front: dtypes");
  const int64_t l = C->dims[0], m = C->dims[1], d = A->dims[1], r = A->dims[2];
  GB_REQUIRE(A->dims[0] == m, "mul_front: bond mismatch");
  GB_REQUIRE(out->dims[0] == l && out->dims[1] == d && out->dims[2] == r, "mul_front: output");
  DevGuard g(ctx->device);
  gemm(ctx, ctx->aux_prec, A->dtype, 'N', 'N', l, d * r, m, 1.0, C->data, l, 0, A->data, m, 0,
       0.0, out->data, l, 0);
  API_END
}

int gb_mps_mul_tail(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* C, gb_tensor* out) {
  API_BEGIN
  for (const gb_tensor* t : {C, A, (const gb_tensor*)out}) check_ctx(t, ctx);
  GB_REQUIRE(C->kind == GB_KIND_BOND && A->kind == GB_KIND_MPS && out->kind == GB_KIND_MPS,
             "mul_tail: kinds");
  GB_REQUIRE(C->dtype == A->dtype && out->dtype == A->dtype, "mul_tail: dtypes");
  const int64_t l = A->dims[0], d = A->dims[1], m = A->dims[2], r = C->dims[1];
  GB_REQUIRE(C->dims[0] == m, "mul_tail: bond mismatch");
  GB_REQUIRE(out->dims[0] == l && out->dims[1] == d && out->dims[2] == r, "mul_tail: output");
  DevGuard g(ctx->device);
  gemm(ctx, ctx->aux_prec, A->dtype, 'N', 'N', l * d, r, m, 1.0, A->data, l * d, 0, C->data, m, 0,
       0.0, out->data, l * d, 0);
  API_END
}

int gb_mps_transfer_bond(gb_ctx* ctx, int side, const gb_tensor* A, const gb_tensor* B,
                         const gb_tensor* X, gb_tensor* out) {
  API_BEGIN
  for (const gb_tensor* t : {A, B, X, (const gb_tensor*)out}) check_ctx(t, ctx);
  GB_REQUIRE(A->kind == GB_KIND_MPS && B->kind == GB_KIND_MPS && X->kind == GB_KIND_BOND &&
                 out->kind == GB_KIND_BOND,
             "transfer_bond: kinds");
  GB_REQUIRE(A->dtype == B->dtype && X->dtype == A->dtype && out->dtype == A->dtype,
             "transfer_bond: dtypes");
  GB_REQUIRE(side == 0 || side == 1, "transfer_bond: side must be 0 (left) or 1 (right)");
  const int dt = A->dtype;
  const int64_t d = A->dims[1];
  GB_REQUIRE(B->dims[1] == d, "transfer_bond: physical dimensions differ");
  DevGuard g(ctx->device);
  const size_t es = elem_size(dt);
  if (side == 0) {
    // out[b, a] = sum_{l l' s} conj(B[l, s, b]) X[l, l'] A[l', s, a]
    const int64_t lB = B->dims[0], lA = A->dims[0], rB = B->dims[2], rA = A->dims[2];
    GB_REQUIRE(X->dims[0] == lB && X->dims[1] == lA && out->dims[0] == rB && out->dims[1] == rA,
               "transfer_bond: shapes");
    void* T = scratch(ctx, SLOT_TMP, (size_t)lB * d * rA * es);
    gemm(ctx, ctx->aux_prec, dt, 'N', 'N', lB, d * rA, lA, 1.0, X->data, lB, 0, A->data, lA, 0,
         0.0, T, lB, 0);  // T = X A : (lB, s, rA)
    gemm(ctx, ctx->aux_prec, dt, 'C', 'N', rB, rA, lB * d, 1.0, B->data, lB * d, 0, T, lB * d, 0,
         0.0, out->data, rB, 0);
  } else {
    // out[a, b] = sum_{s r r'} A[a, s, r] X[r, r'] conj(B[b, s, r'])
    const int64_t lA = A->dims[0], lB = B->dims[0], rA = A->dims[2], rB = B->dims[2];
    GB_REQUIRE(X->dims[0] == rA && X->dims[1] == rB && out->dims[0] == lA && out->dims[1] == lB,
               "transfer_bond: shapes");
    void* T = scratch(ctx, SLOT_TMP, (size_t)lA * d * rB * es);
    gemm(ctx, ctx->aux_prec, dt, 'N', 'N', lA * d, rB, rA, 1.0, A->data, lA * d, 0, X->data, rA,
         0, 0.0, T, lA * d, 0);  // T = A X : (lA, s, rB)
    gemm(ctx, ctx->aux_prec, dt, 'N', 'C', lA, lB, d * rB, 1.0, T, lA, 0, B->data, lB, 0, 0.0,
         out->data, lA, 0);
  }
  API_END
}

int gb_project_complement(gb_ctx* ctx, gb_tensor* Y, const gb_tensor* X) {
  API_BEGIN
  check_ctx(Y, ctx);
  check_ctx(X, ctx);
  GB_REQUIRE(X->kind == GB_KIND_MPS, "project_complement: X must be an MPS tensor");
  GB_REQUIRE(Y->kind == GB_KIND_MPS || Y->kind == GB_KIND_AC2, "project_complement: Y kind");
  GB_REQUIRE(X->dtype == Y->dtype, "project_complement: dtypes");
  const int64_t rows = X->dims[0] * X->dims[1], k = X->dims[2];
  GB_REQUIRE(Y->dims[0] * Y->dims[1] == rows, "project_complement: leading legs mismatch");
  const int64_t cols = numel(Y) / rows;
  DevGuard g(ctx->device);
  const size_t es = elem_size(Y->dtype);
  void* T = scratch(ctx, SLOT_TMP, (size_t)k * cols * es);
  // the auxiliary precision of the context: in split mode Y is itself the output of a
  // split-precision operator, so FP64 here would not add accuracy
  gemm(ctx, ctx->aux_prec, Y->dtype, 'C', 'N', k, cols, rows, 1.0, X->data, rows, 0, Y->data,
       rows, 0, 0.0, T, k, 0);
  gemm(ctx, ctx->aux_prec, Y->dtype, 'N', 'N', rows, cols, k, -1.0, X->data, rows, 0, T, k, 0,
       1.0, Y->data, rows, 0);
  API_END
}

// ---------------------------------------------------------------- gauge
int gb_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, int64_t maxdim, double atol, int normalize,
                 gb_tensor** AL, gb_tensor** S, gb_tensor** AR, double* eps) {
  API_BEGIN
  check_ctx(AC2, ctx);
  GB_REQUIRE(AL && S && AR, "null output");
  GB_REQUIRE(AC2->kind == GB_KIND_AC2, "svd_trunc: input must be a two-site tensor");
  DevGuard g(ctx->device);
  // the Gram route when its singular values decide the truncation, else the SVD below
  if (ctx->svd_method == GB_SVD_GRAM &&
      svd_trunc_gram(ctx, AC2, maxdim, atol, normalize, AL, S, AR, eps))
    return GB_OK;
  const int dt = AC2->dtype;
  const size_t es = elem_size(dt);
  const int64_t Dl = AC2->dims[0], d1 = AC2->dims[1], Dr = AC2->dims[2], d2 = AC2->dims[3];
  const int64_t m = Dl * d1, n = d2 * Dr, k = std::min(m, n);
  // device layout (l, s1, s2, r) is the matrix [(l s1), (s2 r)]
  char* Aw = (char*)scratch(ctx, SLOT_GAUGE, (size_t)m * n * es + 256);
  char* U = (char*)scratch(ctx, SLOT_GAUGE2, (size_t)std::max(m, n) * k * es + 256);
  char* VT = (char*)scratch(ctx, SLOT_GAUGE3, (size_t)k * std::max(m, n) * es + 256);
  double* Sd = (double*)scratch(ctx, SLOT_RED, sizeof(double) * (k + 64) + 4096);
  const bool tall = m >= n;
  if (tall) {
    GB_CHECK_CUDA(cudaMemcpyAsync(Aw, AC2->data, (size_t)m * n * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    svd_tall(ctx, dt, m, n, Aw, U, Sd, VT);  // U m x k, VT k x n
  } else {
    conj_transpose(ctx, dt, m, n, AC2->data, m, Aw, n);  // n x m
    svd_tall(ctx, dt, n, m, Aw, U, Sd, VT);              // U' n x k, VT' k x m
  }
  std::vector<double> hs(k);
  GB_CHECK_CUDA(cudaMemcpyAsync(hs.data(), Sd, sizeof(double) * k, cudaMemcpyDeviceToHost,
                                ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t keep = 0;
  for (int64_t i = 0; i < k; ++i)
    if (hs[i] > atol) ++keep;
  if (maxdim > 0) keep = std::min(keep, maxdim);
  keep = std::max<int64_t>(keep, 1);
  double e2 = 0.0, n2 = 0.0;
  for (int64_t i = keep; i < k; ++i) e2 += hs[i] * hs[i];
  for (int64_t i = 0; i < keep; ++i) n2 += hs[i] * hs[i];
  if (eps) *eps = std::sqrt(e2);
  double scl = normalize ? 1.0 / std::sqrt(n2) : 1.0;
  int64_t dl[3] = {Dl, d1, keep}, dr[3] = {keep, d2, Dr}, dc[2] = {keep, keep};
  gb_tensor* al = new_tensor(ctx, GB_KIND_MPS, dt, 3, dl);
  gb_tensor* ar = new_tensor(ctx, GB_KIND_MPS, dt, 3, dr);
  gb_tensor* sc = new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  if (tall) {
    // AL = U[:, :keep] (m x keep); AR = VT[:keep, :] (keep x n, ld k)
    GB_CHECK_CUDA(cudaMemcpyAsync(al->data, U, (size_t)m * keep * es, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    GB_CHECK_CUDA(cudaMemcpy2DAsync(ar->data, keep * es, VT, k * es, keep * es, n,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    // M = VT'^H S U'^H : AL = (VT'[:keep, :])^H (m x keep), AR = (U'[:, :keep])^H (keep x n)
    conj_transpose(ctx, dt, keep, m, VT, k, al->data, m);
    conj_transpose(ctx, dt, n, keep, U, n, ar->data, keep);
  }
  diag_kernel<<<64, 256, 0, ctx->stream>>>(keep, Sd, scl, (double*)sc->data, is_cplx(dt));
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *AL = al;
  *AR = ar;
  *S = sc;
  API_END
}

// stream-ordered device buffer of a (lane) context
struct StreamBuf {
  gb_ctx* ctx;
  void* p = nullptr;
  StreamBuf(gb_ctx* c, size_t bytes) : ctx(c) {
    GB_CHECK_CUDA(cudaMallocAsync(&p, bytes, c->stream));
  }
  ~StreamBuf() {
    if (p) cudaFreeAsync(p, ctx->stream);
  }
  StreamBuf(const StreamBuf&) = delete;
  StreamBuf& operator=(const StreamBuf&) = delete;
};

int gb_svd_batch(gb_ctx* ctx, int64_t count, const gb_tensor* const* M, gb_tensor** U,
                 gb_tensor** Vh, double* S) {
  API_BEGIN
  GB_REQUIRE(count >= 0 && (count == 0 || (M && U && Vh && S)), "null argument");
  DevGuard g(ctx->device);
  struct Item {
    int64_t m, n;
    size_t soff;
  };
  std::vector<Item> it(count);
  size_t stot = 0;
  for (int64_t i = 0; i < count; ++i) {
    const gb_tensor* t = M[i];
    GB_REQUIRE(t, "null tensor");
    check_ctx(t, ctx);
    GB_REQUIRE(t->kind == GB_KIND_MPS || t->kind == GB_KIND_BOND, "svd_batch: MPS or bond tensors");
    const int64_t n = t->dims[t->ndim - 1], m = numel(t) / std::max<int64_t>(n, 1);
    GB_REQUIRE(m >= n && n > 0, "svd_batch: each matrix must have at least as many rows as columns");
    it[i] = Item{m, n, stot};
    stot += (size_t)n;
    U[i] = Vh[i] = nullptr;
  }
  try {
    for (int64_t i = 0; i < count; ++i) {
      const gb_tensor* t = M[i];
      if (t->kind == GB_KIND_MPS) {
        int64_t du[3] = {t->dims[0], t->dims[1], it[i].n};
        U[i] = new_tensor(ctx, GB_KIND_MPS, t->dtype, 3, du);
      } else {
        int64_t du[2] = {it[i].m, it[i].n};
        U[i] = new_tensor(ctx, GB_KIND_BOND, t->dtype, 2, du);
      }
      int64_t dv[2] = {it[i].n, it[i].n};
      Vh[i] = new_tensor(ctx, GB_KIND_BOND, t->dtype, 2, dv);
    }
    StreamBuf sdev(ctx, stot * sizeof(double) + 256);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    // one factorisation per lane at a time, largest first
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
      return it[a].m * it[a].n * it[a].n > it[b].m * it[b].n * it[b].n;
    });
    run_on_lanes(ctx, count, [&](gb_ctx* L, int64_t oi) {
      const int64_t i = order[oi];
      const gb_tensor* t = M[i];
      StreamBuf A(L, (size_t)it[i].m * it[i].n * elem_size(t->dtype) + 256);
      GB_CHECK_CUDA(cudaMemcpyAsync(A.p, t->data, t->bytes, cudaMemcpyDeviceToDevice, L->stream));
      svd_tall(L, t->dtype, it[i].m, it[i].n, A.p, U[i]->data, (double*)sdev.p + it[i].soff,
               Vh[i]->data);
      GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));
    });
    GB_CHECK_CUDA(cudaMemcpyAsync(S, sdev.p, stot * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    for (int64_t i = 0; i < count; ++i) {
      if (U[i]) free_tensor(U[i]);
      if (Vh[i]) free_tensor(Vh[i]);
      U[i] = Vh[i] = nullptr;
    }
    throw;
  }
  API_END
}

int gb_left_orth(gb_ctx* ctx, const gb_tensor* AC, gb_tensor** AL, gb_tensor** C) {
  API_BEGIN
  check_ctx(AC, ctx);
  GB_REQUIRE(AL && C, "null output");
  GB_REQUIRE(AC->kind == GB_KIND_MPS, "left_orth: input must be an MPS tensor");
  DevGuard g(ctx->device);
  const int dt = AC->dtype;
  const int64_t Dl = AC->dims[0], d = AC->dims[1], Dr = AC->dims[2];
  const int64_t m = Dl * d, n = Dr, k = std::min(m, n);
  int64_t dq[3] = {Dl, d, k}, dc[2] = {k, n};
  gb_tensor* q = new_tensor(ctx, GB_KIND_MPS, dt, 3, dq);
  gb_tensor* r = new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  try {
    qr_pos(ctx, dt, m, n, AC->data, q->data, r->data);
  } catch (...) {
    free_tensor(q);
    free_tensor(r);
    throw;
  }
  *AL = q;
  *C = r;
  API_END
}

int gb_right_orth(gb_ctx* ctx, const gb_tensor* AC, gb_tensor** C, gb_tensor** AR) {
  API_BEGIN
  check_ctx(AC, ctx);
  GB_REQUIRE(AR && C, "null output");
  GB_REQUIRE(AC->kind == GB_KIND_MPS, "right_orth: input must be an MPS tensor");
  DevGuard g(ctx->device);
  const int dt = AC->dtype;
  const size_t es = elem_size(dt);
  const int64_t Dl = AC->dims[0], d = AC->dims[1], Dr = AC->dims[2];
  const int64_t m = Dl, n = d * Dr, k = std::min(m, n);
  // M = L Q  <=>  M^H = Q^H L^H: positive QR of M^H (n x m)
  char* Mh = (char*)scratch(ctx, SLOT_GAUGE2, (size_t)m * n * es + 256);
  conj_transpose(ctx, dt, m, n, AC->data, m, Mh, n);
  char* Qp = (char*)scratch(ctx, SLOT_GAUGE3, (size_t)n * k * es + 256);
  char* Rp = (char*)scratch(ctx, SLOT_KRYLOV_W, (size_t)k * m * es + 256);
  qr_pos(ctx, dt, n, m, Mh, Qp, Rp);  // Qp n x k, Rp k x m
  int64_t dq[3] = {k, d, Dr}, dc[2] = {m, k};
  gb_tensor* q = new_tensor(ctx, GB_KIND_MPS, dt, 3, dq);
  gb_tensor* l = new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  conj_transpose(ctx, dt, n, k, Qp, n, q->data, k);  // AR = Qp^H (k x n)
  conj_transpose(ctx, dt, k, m, Rp, k, l->data, m);  // L = Rp^H (m x k)
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *C = l;
  *AR = q;
  API_END
}

int gb_u1_left_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* q_l, const int32_t* q_s,
                    const int32_t* q_r, gb_tensor** AL, gb_tensor** C, int32_t* q_k,
                    int64_t* k) {
  API_BEGIN
  check_ctx(AC, ctx);
  GB_REQUIRE(AL && C && q_k && k && q_l && q_s && q_r, "null argument");
  GB_REQUIRE(AC->kind == GB_KIND_MPS, "u1_left_orth: input must be an MPS tensor");
  DevGuard g(ctx->device);
  gb::u1_left_orth(ctx, AC, q_l, q_s, q_r, AL, C, q_k, k);
  API_END
}

int gb_u1_right_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* q_l, const int32_t* q_s,
                     const int32_t* q_r, gb_tensor** C, gb_tensor** AR, int32_t* q_k,
                     int64_t* k) {
  API_BEGIN
  check_ctx(AC, ctx);
  GB_REQUIRE(AR && C && q_k && k && q_l && q_s && q_r, "null argument");
  GB_REQUIRE(AC->kind == GB_KIND_MPS, "u1_right_orth: input must be an MPS tensor");
  DevGuard g(ctx->device);
  gb::u1_right_orth(ctx, AC, q_l, q_s, q_r, C, AR, q_k, k);
  API_END
}

int gb_u1_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, const int32_t* q_l, const int32_t* q_s1,
                    const int32_t* q_r, const int32_t* q_s2, int64_t maxdim, double atol,
                    int normalize, gb_tensor** AL, gb_tensor** S, gb_tensor** AR, int32_t* q_k,
                    int64_t* k, double* eps) {
  API_BEGIN
  check_ctx(AC2, ctx);
  GB_REQUIRE(AL && S && AR && q_k && k && q_l && q_s1 && q_s2 && q_r, "null argument");
  GB_REQUIRE(AC2->kind == GB_KIND_AC2, "u1_svd_trunc: input must be a two-site tensor");
  DevGuard g(ctx->device);
  gb::u1_svd_trunc(ctx, AC2, q_l, q_s1, q_s2, q_r, maxdim, atol, normalize, AL, S, AR, q_k, k,
                   eps);
  API_END
}

}  // extern "C"
