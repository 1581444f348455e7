// U(1)-symmetric gauge steps for tensors stored densely with charge-sorted legs.
//
// A U(1)-symmetric tensor here is an ordinary dense device tensor whose entries vanish
// outside the charge-conserving blocks (q_l + q_s = q_r for an MPS tensor), with every
// virtual leg sorted by charge.  The contractions need nothing special: the packed
// operands' nonzero maps let the tensor-core GEMM skip the zero tiles.  What must be
// block-aware are the factorisations: a dense Householder QR or SVD would mix sectors
// (degenerate singular values across sectors are the rule for SU(2)-invariant models) and
// the exact zeros that make the tiles skippable would be lost.  TensorKit factorises a
// symmetric TensorMap block by block (one dense matrix per coupled charge); these routines
// do the same:
//
//   left_orth   AC[l s; r] = AL[l s; k] C[k; r]     per sector c = q_l + q_s = q_r
//   right_orth  AC[l; s r] = C[l; k] AR[k; s r]      per sector c = q_l = q_r - q_s
//   svd_trunc   AC2[l s1; s2 r] ~ AL S AR           per sector, truncation global over
//                                                    sectors (truncrank & trunctol)
//
// Each sector's rows and columns are gathered into a contiguous matrix, factorised with the
// same FP64 routines as the dense path (positive QR, cuSOLVER SVD or the Gram-matrix
// eigendecomposition), and scattered back.  The new bond is sorted by charge; inside a
// sector the kept singular vectors are in descending order.
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>

#include "gb_common.h"

#define CUSOLVER_CHECK_U1(x)                                                          \
  do {                                                                                \
    cusolverStatus_t st_ = (x);                                                       \
    if (st_ != CUSOLVER_STATUS_SUCCESS)                                               \
      throw gb::Error(GB_ERR_CUDA, std::string("cusolver: ") + #x + " -> " +          \
                                       std::to_string((int)st_));                     \
  } while (0)

namespace gb {

// helpers defined in api.cu
gb_tensor* gauge_new_tensor(gb_ctx* ctx, int kind, int dtype, int ndim, const int64_t* dims);
void gauge_free_tensor(gb_tensor* t);
void gauge_qr_pos(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* M, void* Q, void* R);
void gauge_svd_tall(gb_ctx* ctx, int dtype, int64_t m, int64_t n, void* A, void* U, double* S,
                    void* VT);
void gauge_conj_transpose(gb_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A,
                          int64_t lda, void* B, int64_t ldb);
void* gauge_solver(gb_ctx* ctx);

namespace {

// out[i + ni*j] = M[rows[i] + ld*cols[j]]  (scatter: the reverse)
template <bool SCATTER>
__global__ void block_copy_kernel(int64_t ni, int64_t nj, const int64_t* __restrict__ rows,
                                  const int64_t* __restrict__ cols, double* M, int64_t ld,
                                  double* B, int cx) {
  const int64_t n = ni * nj;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % ni, j = e / ni;
    const int64_t src = rows[i] + ld * cols[j];
    if (cx) {
      if (SCATTER) {
        M[2 * src] = B[2 * e];
        M[2 * src + 1] = B[2 * e + 1];
      } else {
        B[2 * e] = M[2 * src];
        B[2 * e + 1] = M[2 * src + 1];
      }
    } else {
      if (SCATTER) M[src] = B[e];
      else B[e] = M[src];
    }
  }
}

// column j of an m x n matrix *= f[j] (or /= f[j])
__global__ void col_scale_kernel(int64_t m, int64_t n, double* __restrict__ A,
                                 const double* __restrict__ f, int divide, int cx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / m;
    const double s = divide ? 1.0 / f[j] : f[j];
    if (cx) {
      A[2 * e] *= s;
      A[2 * e + 1] *= s;
    } else {
      A[e] *= s;
    }
  }
}

// row i of an m x n matrix (ld = m) *= f[i] (or /= f[i])
__global__ void row_scale_kernel(int64_t m, int64_t n, double* __restrict__ A,
                                 const double* __restrict__ f, int divide, int cx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % m;
    const double s = divide ? 1.0 / f[i] : f[i];
    if (cx) {
      A[2 * e] *= s;
      A[2 * e + 1] *= s;
    } else {
      A[e] *= s;
    }
  }
}

// S[o + i, o + i] = v[i] in a k x k matrix
__global__ void put_diag_kernel(int64_t k, int64_t o, int64_t cnt, const double* __restrict__ v,
                                double* __restrict__ S, int cx) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = (o + i) + k * (o + i);
    if (cx) {
      S[2 * e] = v[i];
      S[2 * e + 1] = 0.0;
    } else {
      S[e] = v[i];
    }
  }
}

unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }

// stream-ordered temporary device buffer
struct DevBuf {
  gb_ctx* ctx = nullptr;
  void* p = nullptr;
  DevBuf(gb_ctx* c, size_t bytes) : ctx(c) {
    if (bytes) GB_CHECK_CUDA(cudaMallocAsync(&p, bytes, c->stream));
  }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, ctx->stream);
  }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  template <class T>
  T* as() const {
    return (T*)p;
  }
};

struct Sector {
  int32_t q;
  std::vector<int64_t> rows, cols;
  int64_t ioff = 0;  // offset of rows then cols in the uploaded index table
};

// Sectors present on both sides, ascending charge.  Rows (cols) whose charge has no
// partner carry only zeros of a charge-conserving matrix.
std::vector<Sector> make_sectors(const std::vector<int32_t>& qrow,
                                 const std::vector<int32_t>& qcol) {
  std::map<int32_t, Sector> m;
  for (int64_t i = 0; i < (int64_t)qrow.size(); ++i) m[qrow[i]].rows.push_back(i);
  for (int64_t j = 0; j < (int64_t)qcol.size(); ++j) m[qcol[j]].cols.push_back(j);
  std::vector<Sector> out;
  for (auto& kv : m)
    if (!kv.second.rows.empty() && !kv.second.cols.empty()) {
      kv.second.q = kv.first;
      out.push_back(std::move(kv.second));
    }
  return out;
}

// Sectors in decreasing order of factorisation work (the cube of the smaller side times the
// larger): the lanes take the largest first, so the last sector to start is a small one.
std::vector<int64_t> largest_first(const std::vector<Sector>& ss) {
  std::vector<int64_t> o(ss.size());
  std::iota(o.begin(), o.end(), 0);
  auto work = [&](int64_t c) {
    const double a = (double)ss[c].rows.size(), b = (double)ss[c].cols.size();
    return std::min(a, b) * std::min(a, b) * std::max(a, b);
  };
  std::stable_sort(o.begin(), o.end(), [&](int64_t x, int64_t y) { return work(x) > work(y); });
  return o;
}


// upload every sector's row and column lists into one device table
struct IndexTable {
  DevBuf buf;
  IndexTable(gb_ctx* ctx, std::vector<Sector>& ss) : buf(ctx, table_bytes(ss)) {
    std::vector<int64_t> tab;
    for (auto& s : ss) {
      s.ioff = (int64_t)tab.size();
      tab.insert(tab.end(), s.rows.begin(), s.rows.end());
      tab.insert(tab.end(), s.cols.begin(), s.cols.end());
    }
    if (!tab.empty())
      GB_CHECK_CUDA(cudaMemcpyAsync(buf.p, tab.data(), tab.size() * sizeof(int64_t),
                                    cudaMemcpyHostToDevice, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // tab is a host temporary
  }
  static size_t table_bytes(const std::vector<Sector>& ss) {
    size_t n = 0;
    for (auto& s : ss) n += s.rows.size() + s.cols.size();
    return n * sizeof(int64_t);
  }
  const int64_t* rows(const Sector& s) const { return buf.as<int64_t>() + s.ioff; }
  const int64_t* cols(const Sector& s) const { return rows(s) + s.rows.size(); }
};

void copy_block(gb_ctx* ctx, bool scatter, int64_t ni, int64_t nj, const int64_t* rows,
                const int64_t* cols, void* M, int64_t ld, void* B, bool cx) {
  if (ni == 0 || nj == 0) return;
  if (scatter)
    block_copy_kernel<true><<<blocks_for(ni * nj), 256, 0, ctx->stream>>>(
        ni, nj, rows, cols, (double*)M, ld, (double*)B, cx);
  else
    block_copy_kernel<false><<<blocks_for(ni * nj), 256, 0, ctx->stream>>>(
        ni, nj, rows, cols, (double*)M, ld, (double*)B, cx);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

// device table 0..n-1 (column indices of a contiguous destination range)
struct Iota {
  DevBuf buf;
  Iota(gb_ctx* ctx, int64_t n) : buf(ctx, std::max<int64_t>(n, 1) * sizeof(int64_t)) {
    std::vector<int64_t> v(std::max<int64_t>(n, 1));
    std::iota(v.begin(), v.end(), 0);
    GB_CHECK_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(int64_t),
                                  cudaMemcpyHostToDevice, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  const int64_t* at(int64_t o) const { return buf.as<int64_t>() + o; }
};

// The gathered blocks must hold the whole norm of the input: anything outside them means the
// tensor is not charge-conserving for the given charges.
void check_blocks_norm(gb_ctx* ctx, int dtype, int64_t total_n, const void* M, double blocks_sq) {
  const double full = nrm2(ctx, dtype, total_n, M);
  const double rest = full * full - blocks_sq;
  if (rest > 1e-10 * full * full + 1e-300)
    throw Error(GB_ERR_ARG, "U(1) factorisation: the tensor has weight outside its charge "
                            "blocks (norm^2 " + std::to_string(rest) + ")");
}

void scale_cols(gb_ctx* ctx, int64_t m, int64_t n, void* A, const double* f, bool divide,
                bool cx) {
  if (m == 0 || n == 0) return;
  col_scale_kernel<<<blocks_for(m * n), 256, 0, ctx->stream>>>(m, n, (double*)A, f, divide, cx);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}
void scale_rows_(gb_ctx* ctx, int64_t m, int64_t n, void* A, const double* f, bool divide,
                 bool cx) {
  if (m == 0 || n == 0) return;
  row_scale_kernel<<<blocks_for(m * n), 256, 0, ctx->stream>>>(m, n, (double*)A, f, divide, cx);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}


// Gram route of one sector on a lane: E (g x g) = eigenvectors of the smaller-side Gram
// matrix of M (ni x nj) in descending order, W (g) = its eigenvalues ascending, *info set
void gram_eig_sector(gb_ctx* L, int dt, int64_t ni, int64_t nj, const void* M, void* E, double* W,
                     int* info) {
  const size_t es = elem_size(dt);
  const int64_t g = std::min(ni, nj);
  cusolverDnHandle_t h = (cusolverDnHandle_t)gauge_solver(L);
  const cudaDataType t = is_cplx(dt) ? CUDA_C_64F : CUDA_R_64F;
  DevBuf G(L, (size_t)g * g * es + 256);
  if (ni >= nj)
    gemm_fp64(L, dt, 'C', 'N', g, g, ni, cplx{1, 0}, M, ni, 0, M, ni, 0, cplx{0, 0}, G.p, g, 0, 1);
  else
    gemm_fp64(L, dt, 'N', 'C', g, g, nj, cplx{1, 0}, M, ni, 0, M, ni, 0, cplx{0, 0}, G.p, g, 0, 1);
  (void)h;
  (void)t;
  sym_eig(L, dt, g, G.p, W, info);
  int64_t dims[2] = {g, g}, ins[2] = {1, -g}, outs[2] = {1, g};
  permute(L, dt, 2, dims, G.as<char>() + (size_t)(g - 1) * g * es, ins, E, outs);
  GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));  // hw and the buffers end with this scope
}

}  // namespace

// ------------------------------------------------------------------ Hermitian eigensolver
void sym_eig(gb_ctx* L, int dt, int64_t g, void* G, double* W, int* info) {
  cusolverDnHandle_t h = (cusolverDnHandle_t)gauge_solver(L);
  const bool cx = is_cplx(dt);
  if (L->eig_method == GB_EIG_SYEVJ) {
    // cyclic Jacobi, all on the device (no host stage): tolerance at machine accuracy,
    // eigenvalues ascending like syevd
    GB_REQUIRE(g < (int64_t)1 << 31, "syevj: matrix too large");
    syevjInfo_t p = nullptr;
    CUSOLVER_CHECK_U1(cusolverDnCreateSyevjInfo(&p));
    int lwork = 0;
    try {
      CUSOLVER_CHECK_U1(cusolverDnXsyevjSetMaxSweeps(p, 100));
      if (cx)
        CUSOLVER_CHECK_U1(cusolverDnZheevj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR,
                                                      CUBLAS_FILL_MODE_LOWER, (int)g,
                                                      (cuDoubleComplex*)G, (int)g, W, &lwork, p));
      else
        CUSOLVER_CHECK_U1(cusolverDnDsyevj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR,
                                                      CUBLAS_FILL_MODE_LOWER, (int)g, (double*)G,
                                                      (int)g, W, &lwork, p));
      DevBuf wk(L, (size_t)lwork * elem_size(dt) + 256);
      if (cx)
        CUSOLVER_CHECK_U1(cusolverDnZheevj(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                           (int)g, (cuDoubleComplex*)G, (int)g, W,
                                           wk.as<cuDoubleComplex>(), lwork, info, p));
      else
        CUSOLVER_CHECK_U1(cusolverDnDsyevj(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                           (int)g, (double*)G, (int)g, W, wk.as<double>(), lwork,
                                           info, p));
      count_launch(L);
      GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));
    } catch (...) {
      cusolverDnDestroySyevjInfo(p);
      throw;
    }
    cusolverDnDestroySyevjInfo(p);
    return;
  }
  if (L->eig_method == GB_EIG_SYEVD_DEVICE) {
    // the 32-bit divide-and-conquer interface (no host workspace)
    GB_REQUIRE(g < (int64_t)1 << 31, "syevd: matrix too large");
    int lwork = 0;
    if (cx)
      CUSOLVER_CHECK_U1(cusolverDnZheevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR,
                                                    CUBLAS_FILL_MODE_LOWER, (int)g,
                                                    (cuDoubleComplex*)G, (int)g, W, &lwork));
    else
      CUSOLVER_CHECK_U1(cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR,
                                                    CUBLAS_FILL_MODE_LOWER, (int)g, (double*)G,
                                                    (int)g, W, &lwork));
    DevBuf wk(L, (size_t)lwork * elem_size(dt) + 256);
    if (cx)
      CUSOLVER_CHECK_U1(cusolverDnZheevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                         (int)g, (cuDoubleComplex*)G, (int)g, W,
                                         wk.as<cuDoubleComplex>(), lwork, info));
    else
      CUSOLVER_CHECK_U1(cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                         (int)g, (double*)G, (int)g, W, wk.as<double>(), lwork,
                                         info));
    count_launch(L);
    GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));
    return;
  }
  const cudaDataType t = cx ? CUDA_C_64F : CUDA_R_64F;
  size_t dws = 0, hws = 0;
  CUSOLVER_CHECK_U1(cusolverDnXsyevd_bufferSize(h, (cusolverDnParams_t)L->solver_params,
                                                CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                                g, t, G, g, CUDA_R_64F, W, t, &dws, &hws));
  DevBuf dw(L, dws + 256);
  std::vector<char> hw(hws + 1);
  CUSOLVER_CHECK_U1(cusolverDnXsyevd(h, (cusolverDnParams_t)L->solver_params,
                                     CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, g, t, G, g,
                                     CUDA_R_64F, W, t, dw.p, dws, hw.data(), hws, info));
  count_launch(L);
  GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));  // hw and dw end with this scope
}

// ------------------------------------------------------------------ left_orth
void u1_left_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* ql, const int32_t* qs,
                  const int32_t* qr, gb_tensor** AL, gb_tensor** C, int32_t* qk, int64_t* kout) {
  const int dt = AC->dtype;
  const bool cx = is_cplx(dt);
  const size_t es = elem_size(dt);
  const int64_t Dl = AC->dims[0], d = AC->dims[1], Dr = AC->dims[2];
  const int64_t m = Dl * d;
  std::vector<int32_t> qrow(m), qcol(qr, qr + Dr);
  for (int64_t s = 0; s < d; ++s)
    for (int64_t l = 0; l < Dl; ++l) qrow[l + Dl * s] = ql[l] + qs[s];
  std::vector<Sector> ss = make_sectors(qrow, qcol);
  int64_t k = 0;
  for (auto& s : ss) k += std::min<int64_t>(s.rows.size(), s.cols.size());
  GB_REQUIRE(k > 0, "U(1) left_orth: no charge sector is shared by rows and columns");
  IndexTable tab(ctx, ss);
  Iota iota(ctx, std::max(k, Dr));
  int64_t dl[3] = {Dl, d, k}, dc[2] = {k, Dr};
  gb_tensor* al = gauge_new_tensor(ctx, GB_KIND_MPS, dt, 3, dl);
  gb_tensor* cc = gauge_new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  fill_zero(ctx, al->data, al->bytes);
  fill_zero(ctx, cc->data, cc->bytes);
  std::vector<int64_t> kof(ss.size());
  int64_t ko = 0;
  for (size_t c = 0; c < ss.size(); ++c) {
    const int64_t kc = std::min<int64_t>(ss[c].rows.size(), ss[c].cols.size());
    kof[c] = ko;
    for (int64_t i = 0; i < kc; ++i) qk[ko + i] = ss[c].q;
    ko += kc;
  }
  std::vector<double> nrm(ss.size(), 0.0);
  // sectors are independent: one per lane at a time
  const std::vector<int64_t> order = largest_first(ss);
  run_on_lanes(ctx, (int64_t)ss.size(), [&](gb_ctx* L, int64_t oc) {
    const int64_t c = order[oc];
    const Sector& s = ss[c];
    const int64_t ni = s.rows.size(), nj = s.cols.size(), kc = std::min(ni, nj);
    DevBuf Mb(L, ni * nj * es + 256), Qb(L, ni * kc * es + 256), Rb(L, kc * nj * es + 256);
    copy_block(L, false, ni, nj, tab.rows(s), tab.cols(s), AC->data, m, Mb.p, cx);
    nrm[c] = nrm2(L, dt, ni * nj, Mb.p);
    gauge_qr_pos(L, dt, ni, nj, Mb.p, Qb.p, Rb.p);
    copy_block(L, true, ni, kc, tab.rows(s), iota.at(kof[c]), al->data, m, Qb.p, cx);
    copy_block(L, true, kc, nj, iota.at(kof[c]), tab.cols(s), cc->data, k, Rb.p, cx);
  });
  double blocks_sq = 0.0;
  for (double v : nrm) blocks_sq += v * v;
  check_blocks_norm(ctx, dt, m * Dr, AC->data, blocks_sq);
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *AL = al;
  *C = cc;
  *kout = k;
}

// ------------------------------------------------------------------ right_orth
void u1_right_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* ql, const int32_t* qs,
                   const int32_t* qr, gb_tensor** C, gb_tensor** AR, int32_t* qk, int64_t* kout) {
  const int dt = AC->dtype;
  const bool cx = is_cplx(dt);
  const size_t es = elem_size(dt);
  const int64_t Dl = AC->dims[0], d = AC->dims[1], Dr = AC->dims[2];
  const int64_t n = d * Dr;
  std::vector<int32_t> qrow(ql, ql + Dl), qcol(n);
  for (int64_t r = 0; r < Dr; ++r)
    for (int64_t s = 0; s < d; ++s) qcol[s + d * r] = qr[r] - qs[s];
  std::vector<Sector> ss = make_sectors(qrow, qcol);
  int64_t k = 0;
  for (auto& s : ss) k += std::min<int64_t>(s.rows.size(), s.cols.size());
  GB_REQUIRE(k > 0, "U(1) right_orth: no charge sector is shared by rows and columns");
  IndexTable tab(ctx, ss);
  Iota iota(ctx, std::max(k, Dl));
  int64_t dc[2] = {Dl, k}, dr[3] = {k, d, Dr};
  gb_tensor* cc = gauge_new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  gb_tensor* ar = gauge_new_tensor(ctx, GB_KIND_MPS, dt, 3, dr);
  fill_zero(ctx, ar->data, ar->bytes);
  fill_zero(ctx, cc->data, cc->bytes);
  std::vector<int64_t> kof(ss.size());
  int64_t ko = 0;
  for (size_t c = 0; c < ss.size(); ++c) {
    const int64_t kc = std::min<int64_t>(ss[c].rows.size(), ss[c].cols.size());
    kof[c] = ko;
    for (int64_t i = 0; i < kc; ++i) qk[ko + i] = ss[c].q;
    ko += kc;
  }
  std::vector<double> nrm(ss.size(), 0.0);
  const std::vector<int64_t> order = largest_first(ss);
  run_on_lanes(ctx, (int64_t)ss.size(), [&](gb_ctx* L, int64_t oc) {
    const int64_t c = order[oc];
    const Sector& s = ss[c];
    const int64_t ni = s.rows.size(), nj = s.cols.size(), kc = std::min(ni, nj);
    const size_t blk = ni * nj * es + 256;
    DevBuf Mb(L, blk), Mh(L, blk), Qb(L, blk), Rb(L, blk), Tb(L, blk);
    copy_block(L, false, ni, nj, tab.rows(s), tab.cols(s), AC->data, Dl, Mb.p, cx);
    nrm[c] = nrm2(L, dt, ni * nj, Mb.p);
    // LQ through the positive QR of the adjoint: M^H = Q' R' -> M = R'^H Q'^H
    gauge_conj_transpose(L, dt, ni, nj, Mb.p, ni, Mh.p, nj);
    gauge_qr_pos(L, dt, nj, ni, Mh.p, Qb.p, Rb.p);            // Q' nj x kc, R' kc x ni
    gauge_conj_transpose(L, dt, nj, kc, Qb.p, nj, Tb.p, kc);  // AR block kc x nj
    copy_block(L, true, kc, nj, iota.at(kof[c]), tab.cols(s), ar->data, k, Tb.p, cx);
    gauge_conj_transpose(L, dt, kc, ni, Rb.p, kc, Tb.p, ni);  // C block ni x kc
    copy_block(L, true, ni, kc, tab.rows(s), iota.at(kof[c]), cc->data, Dl, Tb.p, cx);
  });
  double blocks_sq = 0.0;
  for (double v : nrm) blocks_sq += v * v;
  check_blocks_norm(ctx, dt, Dl * n, AC->data, blocks_sq);
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *C = cc;
  *AR = ar;
  *kout = k;
}

// ------------------------------------------------------------------ truncated SVD
void u1_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, const int32_t* ql, const int32_t* qs1,
                  const int32_t* qs2, const int32_t* qr, int64_t maxdim, double atol,
                  int normalize, gb_tensor** AL, gb_tensor** S, gb_tensor** AR, int32_t* qk,
                  int64_t* kout, double* eps) {
  const int dt = AC2->dtype;
  const bool cx = is_cplx(dt);
  const size_t es = elem_size(dt);
  // device layout (l, s1, s2, r); reference dims (l, s1, r, s2)
  const int64_t Dl = AC2->dims[0], d1 = AC2->dims[1], Dr = AC2->dims[2], d2 = AC2->dims[3];
  const int64_t m = Dl * d1, n = d2 * Dr;
  std::vector<int32_t> qrow(m), qcol(n);
  for (int64_t s = 0; s < d1; ++s)
    for (int64_t l = 0; l < Dl; ++l) qrow[l + Dl * s] = ql[l] + qs1[s];
  for (int64_t r = 0; r < Dr; ++r)
    for (int64_t s = 0; s < d2; ++s) qcol[s + d2 * r] = qr[r] - qs2[s];
  std::vector<Sector> ss = make_sectors(qrow, qcol);
  GB_REQUIRE(!ss.empty(), "U(1) svd_trunc: no charge sector is shared by rows and columns");
  IndexTable tab(ctx, ss);
  const bool gram = ctx->svd_method == GB_SVD_GRAM;
  // phase 1: factorise every sector; keep its factors in one arena
  struct Fac {
    int64_t ni, nj, g;
    size_t oM, oU, oV, oS;  // element offsets in the arena (oS: doubles in sig)
  };
  std::vector<Fac> fs(ss.size());
  size_t arena = 0, nsig = 0;
  for (size_t c = 0; c < ss.size(); ++c) {  // the gathered blocks first, contiguous
    Fac& f = fs[c];
    f.ni = ss[c].rows.size();
    f.nj = ss[c].cols.size();
    f.g = std::min(f.ni, f.nj);
    f.oM = arena;
    arena += f.ni * f.nj;
  }
  const size_t blocks_elems = arena;
  for (size_t c = 0; c < ss.size(); ++c) {
    Fac& f = fs[c];
    f.oU = arena;
    arena += gram ? f.g * f.g : f.ni * f.g;
    f.oV = arena;
    arena += gram ? 0 : f.g * f.nj;
    f.oS = nsig;
    nsig += f.g;
  }
  DevBuf ar_(ctx, arena * es + 256), sig(ctx, nsig * sizeof(double) + 256);
  char* base = ar_.as<char>();
  auto at = [&](size_t off) { return (void*)(base + off * es); };
  double blocks_sq = 0.0;
  for (size_t c = 0; c < ss.size(); ++c)
    copy_block(ctx, false, fs[c].ni, fs[c].nj, tab.rows(ss[c]), tab.cols(ss[c]), AC2->data, m,
               at(fs[c].oM), cx);
  {
    const double nb = nrm2(ctx, dt, (int64_t)blocks_elems, at(0));
    blocks_sq = nb * nb;
  }
  DevBuf W(ctx, nsig * sizeof(double) + 256), info(ctx, ss.size() * sizeof(int) + 256);
  // sectors are independent: one per lane at a time
  const std::vector<int64_t> order = largest_first(ss);
  run_on_lanes(ctx, (int64_t)ss.size(), [&](gb_ctx* L, int64_t oc) {
    const int64_t c = order[oc];
    const Fac& f = fs[c];
    void* Mc = at(f.oM);
    double* sc = sig.as<double>() + f.oS;
    if (gram) {
      gram_eig_sector(L, dt, f.ni, f.nj, Mc, at(f.oU), W.as<double>() + f.oS, info.as<int>() + c);
      return;
    }
    const size_t blk = f.ni * f.nj * es + 256;
    DevBuf W1(L, blk), W2(L, blk), W3(L, blk);
    if (f.ni >= f.nj) {
      GB_CHECK_CUDA(cudaMemcpyAsync(W1.p, Mc, f.ni * f.nj * es, cudaMemcpyDeviceToDevice,
                                    L->stream));
      gauge_svd_tall(L, dt, f.ni, f.nj, W1.p, at(f.oU), sc, at(f.oV));
    } else {
      // SVD of M^H (tall): M^H = U' S VT' -> M = VT'^H S U'^H
      gauge_conj_transpose(L, dt, f.ni, f.nj, Mc, f.ni, W1.p, f.nj);
      gauge_svd_tall(L, dt, f.nj, f.ni, W1.p, W2.p, sc, W3.p);  // U' nj x g, VT' g x ni
      gauge_conj_transpose(L, dt, f.g, f.ni, W3.p, f.g, at(f.oU), f.ni);  // U = VT'^H
      gauge_conj_transpose(L, dt, f.nj, f.g, W2.p, f.nj, at(f.oV), f.g);  // VT = U'^H
    }
    GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));
  });
  if (gram) {
    // singular values from the Gram eigenvalues (ascending per sector), descending
    std::vector<int> hinfo(ss.size());
    std::vector<double> hW(nsig), hsig(nsig);
    GB_CHECK_CUDA(cudaMemcpyAsync(hinfo.data(), info.p, ss.size() * sizeof(int),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(hW.data(), W.p, nsig * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t c = 0; c < ss.size(); ++c) {
      if (hinfo[c] != 0) throw Error(GB_ERR_CUDA, "syevd info = " + std::to_string(hinfo[c]));
      const Fac& f = fs[c];
      for (int64_t q = 0; q < f.g; ++q)
        hsig[f.oS + q] = std::sqrt(std::max(hW[f.oS + f.g - 1 - q], 0.0));
    }
    GB_CHECK_CUDA(cudaMemcpyAsync(sig.p, hsig.data(), nsig * sizeof(double),
                                  cudaMemcpyHostToDevice, ctx->stream));
  }
  check_blocks_norm(ctx, dt, m * n, AC2->data, blocks_sq);
  // phase 2: global truncation (truncrank & trunctol over all sectors)
  std::vector<double> hs(nsig);
  GB_CHECK_CUDA(cudaMemcpyAsync(hs.data(), sig.p, nsig * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  struct SV {
    double s;
    int c;
    int64_t j;
  };
  std::vector<SV> all;
  all.reserve(nsig);
  for (size_t c = 0; c < ss.size(); ++c)
    for (int64_t j = 0; j < fs[c].g; ++j) all.push_back({hs[fs[c].oS + j], (int)c, j});
  std::stable_sort(all.begin(), all.end(), [](const SV& a, const SV& b) {
    if (a.s != b.s) return a.s > b.s;
    if (a.c != b.c) return a.c < b.c;
    return a.j < b.j;
  });
  int64_t keep = 0;
  for (auto& v : all)
    if (v.s > atol) ++keep;
  if (maxdim > 0) keep = std::min(keep, maxdim);
  keep = std::max<int64_t>(keep, 1);
  if (gram) {
    // Gram singular values carry an absolute error of about eps_mach * s_max^2 / s with
    // s_max the largest value of their own block: below 1e-7 s_max they are rounding noise.
    // When a kept value or the first discarded one is that small, the rank and the discarded
    // weight cannot be read off them: factorise every block by its SVD instead.
    auto resolved = [&](const SV& v) { return v.s >= 1e-7 * hs[fs[v.c].oS]; };
    if (!resolved(all[keep - 1]) || (keep < (int64_t)all.size() && !resolved(all[keep]))) {
      const int saved = ctx->svd_method;
      ctx->svd_method = GB_SVD_GESVD;
      try {
        u1_svd_trunc(ctx, AC2, ql, qs1, qs2, qr, maxdim, atol, normalize, AL, S, AR, qk, kout,
                     eps);
      } catch (...) {
        ctx->svd_method = saved;
        throw;
      }
      ctx->svd_method = saved;
      return;
    }
  }
  double e2 = 0.0;
  for (size_t i = keep; i < all.size(); ++i) e2 += all[i].s * all[i].s;
  if (eps) *eps = std::sqrt(e2);
  std::vector<int64_t> kc(ss.size(), 0);
  for (int64_t i = 0; i < keep; ++i) kc[all[i].c]++;  // the largest kc of each sector
  if (gram) GB_REQUIRE(all[keep - 1].s > 0.0, "U(1) svd_trunc (Gram): a kept singular value is zero");
  // phase 3: assemble AL (Dl, d1, k), C (k, k), AR (k, d2, Dr) with the new bond by charge
  const int64_t k = keep;
  int64_t dl[3] = {Dl, d1, k}, dr[3] = {k, d2, Dr}, dc[2] = {k, k};
  gb_tensor* al = gauge_new_tensor(ctx, GB_KIND_MPS, dt, 3, dl);
  gb_tensor* ar = gauge_new_tensor(ctx, GB_KIND_MPS, dt, 3, dr);
  gb_tensor* cc = gauge_new_tensor(ctx, GB_KIND_BOND, dt, 2, dc);
  fill_zero(ctx, al->data, al->bytes);
  fill_zero(ctx, ar->data, ar->bytes);
  fill_zero(ctx, cc->data, cc->bytes);
  Iota iota(ctx, k);
  std::vector<int64_t> kof(ss.size(), 0), kept;
  int64_t ko = 0;
  for (size_t c = 0; c < ss.size(); ++c) {
    kof[c] = ko;
    if (kc[c] == 0) continue;
    kept.push_back((int64_t)c);
    for (int64_t i = 0; i < kc[c]; ++i) qk[ko + i] = ss[c].q;
    ko += kc[c];
  }
  GB_TRACE(ctx);  // host-side truncation and output set-up end here
  {
    const std::vector<int64_t> order = largest_first(ss);
    std::vector<int64_t> rank(ss.size());
    for (size_t i = 0; i < order.size(); ++i) rank[order[i]] = (int64_t)i;
    std::stable_sort(kept.begin(), kept.end(),
                     [&](int64_t x, int64_t y) { return rank[x] < rank[y]; });
  }
  run_on_lanes(ctx, (int64_t)kept.size(), [&](gb_ctx* L, int64_t idx) {
    const size_t c = (size_t)kept[idx];
    const Fac& f = fs[c];
    const int64_t kk = kc[c], o = kof[c];
    const Sector& s = ss[c];
    const double* sc = sig.as<double>() + f.oS;
    const size_t blk = std::max(f.ni, f.nj) * std::max<int64_t>(kk, f.g) * es + 256;
    DevBuf W1(L, blk), W2(L, blk), W3(L, blk);
    if (!gram) {
      copy_block(L, true, f.ni, kk, tab.rows(s), iota.at(o), al->data, m, at(f.oU), cx);
      // rows 0..kk-1 of VT (g x nj, ld g): gather them contiguously first
      gauge_conj_transpose(L, dt, f.g, f.nj, at(f.oV), f.g, W1.p, f.nj);  // V  nj x g
      gauge_conj_transpose(L, dt, f.nj, kk, W1.p, f.nj, W2.p, kk);       // VT_k kk x nj
      copy_block(L, true, kk, f.nj, iota.at(o), tab.cols(s), ar->data, k, W2.p, cx);
      put_diag_kernel<<<blocks_for(kk), 256, 0, L->stream>>>(k, o, kk, sc, (double*)cc->data, cx);
      GB_CHECK_CUDA(cudaGetLastError());
      count_launch(L);
    } else if (f.ni >= f.nj) {
      // E (nj x kk) eigenvectors; U = M E / sigma -> Q R; AL = Q, C = R Sigma, AR = E^H
      void* E = at(f.oU);
      gemm_fp64(L, dt, 'N', 'N', f.ni, kk, f.nj, cplx{1, 0}, at(f.oM), f.ni, 0, E, f.nj, 0,
                cplx{0, 0}, W1.p, f.ni, 0, 1);
      scale_cols(L, f.ni, kk, W1.p, sc, true, cx);
      gauge_qr_pos(L, dt, f.ni, kk, W1.p, W2.p, W3.p);  // Q ni x kk, R kk x kk
      scale_cols(L, kk, kk, W3.p, sc, false, cx);       // R Sigma
      copy_block(L, true, f.ni, kk, tab.rows(s), iota.at(o), al->data, m, W2.p, cx);
      copy_block(L, true, kk, kk, iota.at(o), iota.at(o), cc->data, k, W3.p, cx);
      gauge_conj_transpose(L, dt, f.nj, kk, E, f.nj, W1.p, kk);  // E^H kk x nj
      copy_block(L, true, kk, f.nj, iota.at(o), tab.cols(s), ar->data, k, W1.p, cx);
    } else {
      // E (ni x kk); AL = E; W = Sigma^-1 E^H M -> L Q; AR = Q, C = Sigma L
      void* E = at(f.oU);
      copy_block(L, true, f.ni, kk, tab.rows(s), iota.at(o), al->data, m, E, cx);
      gemm_fp64(L, dt, 'C', 'N', kk, f.nj, f.ni, cplx{1, 0}, E, f.ni, 0, at(f.oM), f.ni, 0,
                cplx{0, 0}, W1.p, kk, 0, 1);
      scale_rows_(L, kk, f.nj, W1.p, sc, true, cx);
      gauge_conj_transpose(L, dt, kk, f.nj, W1.p, kk, W2.p, f.nj);  // W^H nj x kk
      gauge_qr_pos(L, dt, f.nj, kk, W2.p, W3.p, W1.p);               // Q' nj x kk, R' kk x kk
      gauge_conj_transpose(L, dt, f.nj, kk, W3.p, f.nj, W2.p, kk);  // AR block = Q'^H
      copy_block(L, true, kk, f.nj, iota.at(o), tab.cols(s), ar->data, k, W2.p, cx);
      gauge_conj_transpose(L, dt, kk, kk, W1.p, kk, W3.p, kk);      // L = R'^H
      scale_rows_(L, kk, kk, W3.p, sc, false, cx);                   // Sigma L
      copy_block(L, true, kk, kk, iota.at(o), iota.at(o), cc->data, k, W3.p, cx);
    }
    GB_CHECK_CUDA(cudaStreamSynchronize(L->stream));
  });
  if (normalize) {
    const double nc = nrm2(ctx, dt, k * k, cc->data);
    scale(ctx, dt, k * k, cplx{1.0 / nc, 0}, cc->data);
  }
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  *AL = al;
  *AR = ar;
  *S = cc;
  *kout = k;
}

}  // namespace gb
