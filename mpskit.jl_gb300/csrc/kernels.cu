// Memory-bound and CUDA-core kernels of libmpsgb: strided permutes, the sparse
// "mode mix" that applies small MPO-derived matrices along tensor legs, delta-term
// additions, the FP64/complex SIMT GEMM of the plain-precision path, and the
// BLAS-1 / Krylov reductions (warp-shuffle tree reductions, two-pass, deterministic).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "gb_common.h"

namespace gb {

// ------------------------------------------------------------------ complex helpers
struct dcx {
  double re, im;
};
__host__ __device__ inline dcx mk(double r, double i) { return dcx{r, i}; }
__device__ inline dcx cadd(dcx a, dcx b) { return mk(a.re + b.re, a.im + b.im); }
__device__ inline dcx cmul(dcx a, dcx b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ inline dcx cconj(dcx a) { return mk(a.re, -a.im); }
__device__ inline dcx cfma(dcx a, dcx b, dcx c) {  // a*b + c
  return mk(fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im)));
}

template <typename T>
struct Ops;
template <>
struct Ops<double> {
  static __device__ double zero() { return 0.0; }
  static __device__ double fmaop(double a, double b, double c) { return fma(a, b, c); }
  static __device__ double conj(double a) { return a; }
  static __device__ double mul(double a, double b) { return a * b; }
  static __device__ double add(double a, double b) { return a + b; }
  static __device__ double from(cplx c) { return c.re; }
  static __device__ bool is_zero(double a) { return a == 0.0; }
};
template <>
struct Ops<dcx> {
  static __device__ dcx zero() { return mk(0, 0); }
  static __device__ dcx fmaop(dcx a, dcx b, dcx c) { return cfma(a, b, c); }
  static __device__ dcx conj(dcx a) { return cconj(a); }
  static __device__ dcx mul(dcx a, dcx b) { return cmul(a, b); }
  static __device__ dcx add(dcx a, dcx b) { return cadd(a, b); }
  static __device__ dcx from(cplx c) { return mk(c.re, c.im); }
  static __device__ bool is_zero(dcx a) { return a.re == 0.0 && a.im == 0.0; }
};

static inline unsigned nblocks(int64_t n, int bs, int64_t cap = 1 << 20) {
  int64_t b = (n + bs - 1) / bs;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

#define LAUNCH_CHECK() GB_CHECK_CUDA(cudaGetLastError())

// ------------------------------------------------------------------ permute
struct PermArgs {
  int nd;
  int64_t dims[6];
  int64_t is[6];
  int64_t os[6];
  int64_t total;
};

template <typename T>
__global__ void permute_kernel(PermArgs p, const T* __restrict__ in, T* __restrict__ out) {
  for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < p.total;
       lin += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = lin, io = 0, oo = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d) {
      if (d < p.nd) {
        int64_t q = r % p.dims[d];
        r /= p.dims[d];
        io += q * p.is[d];
        oo += q * p.os[d];
      }
    }
    out[oo] = in[io];
  }
}

void permute(gb_ctx* ctx, int dtype, int nd, const int64_t* dims, const void* in,
             const int64_t* in_strides, void* out, const int64_t* out_strides) {
  PermArgs p{};
  p.nd = nd;
  p.total = 1;
  for (int i = 0; i < nd; ++i) {
    p.dims[i] = dims[i];
    p.is[i] = in_strides[i];
    p.os[i] = out_strides[i];
    p.total *= dims[i];
  }
  if (p.total == 0) return;
  unsigned nb = nblocks(p.total, 256, 152 * 32);
  if (is_cplx(dtype))
    permute_kernel<dcx><<<nb, 256, 0, ctx->stream>>>(p, (const dcx*)in, (dcx*)out);
  else
    permute_kernel<double><<<nb, 256, 0, ctx->stream>>>(p, (const double*)in, (double*)out);
  LAUNCH_CHECK();
  count_launch(ctx);
}

// ------------------------------------------------------------------ sparse mode mix
template <typename T>
__global__ void mix_kernel(int64_t A, int64_t N, int64_t xa, int64_t xn, int64_t ya, int64_t yn,
                           const int64_t* __restrict__ in_off, const int64_t* __restrict__ out_off,
                           const int* __restrict__ row_ptr, const int* __restrict__ col,
                           const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y,
                           double beta) {
  const int J = blockIdx.y;
  const int e0 = row_ptr[J], e1 = row_ptr[J + 1];
  const int64_t yo = out_off[J];
  for (int64_t n = blockIdx.z; n < N; n += gridDim.z) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < A;
         a += (int64_t)gridDim.x * blockDim.x) {
      T acc = Ops<T>::zero();
      const int64_t xb = a * xa + n * xn;
      for (int e = e0; e < e1; ++e) acc = Ops<T>::fmaop(val[e], x[xb + in_off[col[e]]], acc);
      T* yp = y + a * ya + yo + n * yn;
      if (beta != 0.0) {
        T old = *yp;
        if constexpr (sizeof(T) == 8) {
          acc = acc + beta * old;
        } else {
          acc = Ops<T>::add(acc, mk(beta * old.re, beta * old.im));
        }
      }
      *yp = acc;
    }
  }
}

MixDev mix_upload(gb_ctx* ctx, const MixPlan& p) {
  MixDev m;
  m.A = p.A;
  m.N = p.N;
  m.nJ = p.nJ;
  m.xa = p.xa;
  m.xn = p.xn;
  m.ya = p.ya;
  m.yn = p.yn;
  m.cplx = p.cplx;
  GB_REQUIRE((int64_t)p.out_off.size() == p.nJ, "mix plan: out_off size");
  GB_REQUIRE((int64_t)p.row_ptr.size() == p.nJ + 1, "mix plan: row_ptr size");
  size_t nnz = p.col.size();
  size_t vsz = (p.cplx ? 2 : 1) * std::max<size_t>(nnz, 1);
  size_t b0 = sizeof(int64_t) * std::max<size_t>(p.in_off.size(), 1);
  size_t b1 = sizeof(int64_t) * std::max<size_t>(p.out_off.size(), 1);
  size_t b2 = sizeof(int) * p.row_ptr.size();
  size_t b3 = sizeof(int) * std::max<size_t>(nnz, 1);
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  size_t tot = al(sizeof(double) * vsz) + al(b0) + al(b1) + al(b2) + al(b3);
  std::vector<char> host(tot, 0);
  size_t o = 0;
  size_t oval = o;
  if (!p.val.empty()) memcpy(host.data() + o, p.val.data(), sizeof(double) * p.val.size());
  o += al(sizeof(double) * vsz);
  size_t oin = o;
  if (!p.in_off.empty()) memcpy(host.data() + o, p.in_off.data(), b0);
  o += al(b0);
  size_t oout = o;
  if (!p.out_off.empty()) memcpy(host.data() + o, p.out_off.data(), b1);
  o += al(b1);
  size_t orp = o;
  memcpy(host.data() + o, p.row_ptr.data(), b2);
  o += al(b2);
  size_t ocol = o;
  if (nnz) memcpy(host.data() + o, p.col.data(), sizeof(int) * nnz);
  void* d = nullptr;
  GB_CHECK_CUDA(cudaMalloc(&d, tot));
  GB_CHECK_CUDA(cudaMemcpyAsync(d, host.data(), tot, cudaMemcpyHostToDevice, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  m.buf = d;
  m.bytes = tot;
  m.val = (const double*)((char*)d + oval);
  m.in_off = (const int64_t*)((char*)d + oin);
  m.out_off = (const int64_t*)((char*)d + oout);
  m.row_ptr = (const int*)((char*)d + orp);
  m.col = (const int*)((char*)d + ocol);
  return m;
}

void mix_free(MixDev& m) {
  if (m.buf) cudaFree(m.buf);
  m.buf = nullptr;
}

void mix_run(gb_ctx* ctx, const MixDev& m, int dtype, const void* x, void* y, double beta) {
  if (m.nJ == 0 || m.A == 0 || m.N == 0) return;
  GB_REQUIRE(m.nJ <= 65535, "mix: too many output rows");
  dim3 grid(nblocks(m.A, 128, 64), (unsigned)m.nJ, (unsigned)std::min<int64_t>(m.N, 65535));
  if (is_cplx(dtype)) {
    GB_REQUIRE(m.cplx, "mix: complex data needs complex coefficients");
    mix_kernel<dcx><<<grid, 128, 0, ctx->stream>>>(m.A, m.N, m.xa, m.xn, m.ya, m.yn, m.in_off,
                                                   m.out_off, m.row_ptr, m.col, (const dcx*)m.val,
                                                   (const dcx*)x, (dcx*)y, beta);
  } else {
    GB_REQUIRE(!m.cplx, "mix: real data needs real coefficients");
    mix_kernel<double><<<grid, 128, 0, ctx->stream>>>(m.A, m.N, m.xa, m.xn, m.ya, m.yn, m.in_off,
                                                      m.out_off, m.row_ptr, m.col, m.val,
                                                      (const double*)x, (double*)y, beta);
  }
  LAUNCH_CHECK();
  count_launch(ctx);
}

// ------------------------------------------------------------------ diagonal additions
template <typename T>
__global__ void add_diag_kernel(T* y, const int64_t* offs, const T* vals, int nJ, int64_t count,
                                int64_t ds) {
  int J = blockIdx.y;
  T v = vals[J];
  int64_t o = offs[J];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    y[o + i * ds] = Ops<T>::add(y[o + i * ds], v);
}

void add_diag(gb_ctx* ctx, int dtype, void* y, const std::vector<int64_t>& offs,
              const std::vector<double>& vals, int64_t count, int64_t ds) {
  int nJ = (int)offs.size();
  if (nJ == 0 || count == 0) return;
  size_t vb = vals.size() * sizeof(double);
  size_t ob = offs.size() * sizeof(int64_t);
  char* d = (char*)scratch(ctx, SLOT_TMP2, vb + ob + 256);
  GB_CHECK_CUDA(cudaMemcpyAsync(d, vals.data(), vb, cudaMemcpyHostToDevice, ctx->stream));
  char* doff = d + ((vb + 255) & ~size_t(255));
  GB_CHECK_CUDA(cudaMemcpyAsync(doff, offs.data(), ob, cudaMemcpyHostToDevice, ctx->stream));
  dim3 grid(nblocks(count, 256, 64), nJ);
  if (is_cplx(dtype))
    add_diag_kernel<dcx><<<grid, 256, 0, ctx->stream>>>((dcx*)y, (const int64_t*)doff,
                                                        (const dcx*)d, nJ, count, ds);
  else
    add_diag_kernel<double><<<grid, 256, 0, ctx->stream>>>((double*)y, (const int64_t*)doff,
                                                           (const double*)d, nJ, count, ds);
  LAUNCH_CHECK();
  count_launch(ctx);
  // the tables live in a scratch slot: finish before the slot can be reused
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ------------------------------------------------------------------ FP64 SIMT GEMM
// 64x64 output tile, 256 threads, 4x4 register tile per thread, BK = 16.
constexpr int GBM = 64, GBN = 64, GBK = 16;

template <typename T>
__device__ inline T load_op(const T* __restrict__ P, int64_t ld, char op, int64_t r, int64_t c,
                            int64_t R, int64_t Cn) {
  // element (r, c) of op(P) where op(P) is R x Cn
  if (r >= R || c >= Cn) return Ops<T>::zero();
  if (op == 'N') return P[r + ld * c];
  T v = P[c + ld * r];
  return op == 'C' ? Ops<T>::conj(v) : v;
}

// Nonzero map of op(P) (R x Cn) at 64 x 64 granularity: bit (r / 64, c / 64) of
// mask[(tile) * kw + word] where the tile index runs along `tile_dim` (0: rows, 1: cols) and
// the 64-wide block index along the other dimension.  One CTA per 64 x 64 region.
template <typename T>
__global__ void zero_map_kernel(char op, const T* __restrict__ P, int64_t ld, int64_t stride,
                                int64_t R, int64_t Cn, int tile_dim, uint32_t* __restrict__ mask,
                                int kw, int64_t mstride) {
  const int64_t b = blockIdx.z;
  P += b * stride;
  const int64_t r0 = (int64_t)blockIdx.x * 64, c0 = (int64_t)blockIdx.y * 64;
  const bool rowfast = (op == 'N');
  int nz = 0;
  for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
    const int fast = e % 64, slow = e / 64;
    const int64_t r = r0 + (rowfast ? fast : slow), c = c0 + (rowfast ? slow : fast);
    if (r < R && c < Cn) {
      const T v = rowfast ? P[r + ld * c] : P[c + ld * r];
      nz |= !Ops<T>::is_zero(v);
    }
  }
  if (__syncthreads_or(nz) && threadIdx.x == 0) {
    const int64_t tile = tile_dim == 0 ? blockIdx.x : blockIdx.y;
    const int64_t kb = tile_dim == 0 ? blockIdx.y : blockIdx.x;
    atomicOr(&mask[b * mstride + tile * kw + kb / 32], 1u << (kb % 32));
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    gemm_simt_kernel(char opA, char opB, int64_t M, int64_t N, int64_t K, T alpha,
                     const T* __restrict__ A, int64_t lda, int64_t sA, const T* __restrict__ B,
                     int64_t ldb, int64_t sB, T beta, bool use_beta, T* __restrict__ C,
                     int64_t ldc, int64_t sC, const uint32_t* __restrict__ mA,
                     const uint32_t* __restrict__ mB, int kw, int64_t mAb, int64_t mBb,
                     int64_t kchunk) {
  __shared__ T As[GBK][GBM + 1];
  __shared__ T Bs[GBK][GBN + 1];
  // kchunk > 0: split K (batch 1): slice z covers k in [z kchunk, (z + 1) kchunk) and writes
  // its partial product to C + z sC (no beta); the slices are summed by a reduction kernel
  const int64_t bz = blockIdx.z;
  const int64_t kbeg = kchunk ? bz * kchunk : 0;
  const int64_t kend = kchunk ? min(K, kbeg + kchunk) : K;
  if (!kchunk) {
    A += bz * sA;
    B += bz * sB;
  }
  C += bz * sC;
  const int64_t m0 = (int64_t)blockIdx.x * GBM, n0 = (int64_t)blockIdx.y * GBN;
  const int tid = threadIdx.x;
  const int tm = (tid % 16) * 4, tn = (tid / 16) * 4;
  // zero-tile skipping: 64-wide k-blocks in which this A row tile or B column tile is zero
  const int64_t bm = kchunk ? 0 : bz;
  const uint32_t* ma = mA ? mA + (sA ? bm : 0) * mAb + (int64_t)blockIdx.x * kw : nullptr;
  const uint32_t* mb = mB ? mB + (sB ? bm : 0) * mBb + (int64_t)blockIdx.y * kw : nullptr;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = Ops<T>::zero();
  for (int64_t k0 = kbeg; k0 < kend; k0 += GBK) {
    if (ma) {
      const int64_t kb = k0 / 64;
      if (!((ma[kb / 32] & mb[kb / 32]) >> (kb % 32) & 1u)) {
        k0 = (kb + 1) * 64 - GBK;  // the loop increment lands on the next 64-block
        continue;
      }
    }
    // A tile: GBM x GBK = 1024 elements, 4 per thread
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      int e = tid + 256 * l;
      int r, c;
      if (opA == 'N') {
        r = e % GBM;
        c = e / GBM;
      } else {
        c = e % GBK;
        r = e / GBK;
      }
      As[c][r] = load_op(A, lda, opA, m0 + r, k0 + c, M, kend);
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      int e = tid + 256 * l;
      int r, c;  // r = k index, c = n index
      if (opB == 'N') {
        r = e % GBK;
        c = e / GBK;
      } else {
        c = e % GBN;
        r = e / GBN;
      }
      Bs[r][c] = load_op(B, ldb, opB, k0 + r, n0 + c, kend, N);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = Ops<T>::fmaop(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    int64_t n = n0 + tn + j;
    if (n >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t m = m0 + tm + i;
      if (m >= M) continue;
      T v = Ops<T>::mul(alpha, acc[i][j]);
      if (use_beta) v = Ops<T>::fmaop(beta, C[m + ldc * n], v);
      C[m + ldc * n] = v;
    }
  }
}

// C = beta C + sum_z W[z] over the split-K slices, summed in slice order (deterministic)
template <typename T>
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int nsplit, const T* __restrict__ W,
                                     T beta, bool use_beta, T* __restrict__ C, int64_t ldc) {
  const int64_t MN = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN;
       e += (int64_t)gridDim.x * blockDim.x) {
    T v = W[e];
    for (int z = 1; z < nsplit; ++z) v = Ops<T>::add(v, W[(int64_t)z * MN + e]);
    const int64_t m = e % M, n = e / M;
    if (use_beta) v = Ops<T>::fmaop(beta, C[m + ldc * n], v);
    C[m + ldc * n] = v;
  }
}

void gemm_fp64(gb_ctx* ctx, int dtype, char opA, char opB, int64_t M, int64_t N, int64_t K,
               cplx alpha, const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb,
               int64_t sB, cplx beta, void* C, int64_t ldc, int64_t sC, int64_t batch) {
  if (M == 0 || N == 0 || batch == 0) return;
  GB_REQUIRE(batch <= 65535, "gemm: batch too large");
  GB_REQUIRE((N + GBN - 1) / GBN <= 65535, "gemm: N too large");
  dim3 grid((unsigned)((M + GBM - 1) / GBM), (unsigned)((N + GBN - 1) / GBN), (unsigned)batch);
  bool use_beta = (beta.re != 0.0 || beta.im != 0.0);
  if (K == 0) {
    // C = beta*C
    GB_REQUIRE(batch == 1 && ldc == M, "gemm: K == 0 only for dense C");
    if (!use_beta) {
      fill_zero(ctx, C, (size_t)M * N * elem_size(dtype));
    } else {
      scale(ctx, dtype, M * N, beta, C);
    }
    return;
  }
  // large products skip zero 64 x 64 x 64 blocks (block-sparse operands stored densely)
  uint32_t* masks = nullptr;
  const int kw = (int)((K + 64 * 32 - 1) / (64 * 32));
  const int64_t mt = grid.x, nt = grid.y;
  const int64_t bA = sA ? batch : 1, bB = sB ? batch : 1;
  // (the grouped schedule only changes split-precision operators with known sectors: the
  // FP64 GEMM keeps its block skipping under it)
  const bool skip = (ctx->gemm_schedule == GB_SCHED_PERSISTENT ||
                     ctx->gemm_schedule == GB_SCHED_GROUPED) &&
                    (double)M * (double)N * (double)K >= 1.3e8 && (K + 63) / 64 <= 65535;
  if (skip) {
    const size_t words = (size_t)(bA * mt + bB * nt) * kw;
    GB_CHECK_CUDA(cudaMallocAsync((void**)&masks, words * 4, ctx->stream));
    GB_CHECK_CUDA(cudaMemsetAsync(masks, 0, words * 4, ctx->stream));
    const int64_t kb = (K + 63) / 64;
    dim3 ga((unsigned)mt, (unsigned)kb, (unsigned)bA), gb_((unsigned)kb, (unsigned)nt, (unsigned)bB);
    uint32_t* mB = masks + bA * mt * kw;
    if (is_cplx(dtype)) {
      zero_map_kernel<dcx><<<ga, 256, 0, ctx->stream>>>(opA, (const dcx*)A, lda, sA, M, K, 0,
                                                        masks, kw, mt * kw);
      zero_map_kernel<dcx><<<gb_, 256, 0, ctx->stream>>>(opB, (const dcx*)B,
                                                         ldb, sB, K, N, 1, mB, kw, nt * kw);
    } else {
      zero_map_kernel<double><<<ga, 256, 0, ctx->stream>>>(opA, (const double*)A, lda, sA, M, K,
                                                           0, masks, kw, mt * kw);
      zero_map_kernel<double><<<gb_, 256, 0, ctx->stream>>>(opB, (const double*)B, ldb, sB, K,
                                                            N, 1, mB, kw, nt * kw);
    }
    LAUNCH_CHECK();
    count_launch_n(ctx, 2);
  }
  const uint32_t* mA_ = masks;
  const uint32_t* mB_ = masks ? masks + bA * mt * kw : nullptr;
  // a grid that fills less than half the GPU splits K over more CTAs (FP64 runs at a few
  // operations per clock per SM on GB300: every SM has to take part); slices of at least 128
  // (a multiple of the 64-wide zero-block granularity), summed in order by a second kernel.
  // Not on lane contexts: their GEMMs run concurrently and fill the GPU together.
  int nsplit = 1;
  const int64_t tiles = mt * nt;
  if (batch == 1 && !ctx->lane && ctx->num_sms > 0 && tiles * 2 <= ctx->num_sms && K >= 256) {
    nsplit = (int)std::min<int64_t>({(int64_t)ctx->num_sms / tiles, K / 128, 16});
    if (nsplit < 2) nsplit = 1;
  }
  const size_t es = elem_size(dtype);
  if (nsplit > 1) {
    const int64_t kchunk = ((K + nsplit - 1) / nsplit + 63) / 64 * 64;
    nsplit = (int)((K + kchunk - 1) / kchunk);
    void* W = scratch(ctx, SLOT_SPLITK, (size_t)nsplit * M * N * es);
    dim3 gs(grid.x, grid.y, (unsigned)nsplit);
    const unsigned rb = (unsigned)std::min<int64_t>((M * N + 255) / 256, 4096);
    if (is_cplx(dtype)) {
      gemm_simt_kernel<dcx><<<gs, 256, 0, ctx->stream>>>(
          opA, opB, M, N, K, mk(alpha.re, alpha.im), (const dcx*)A, lda, 0, (const dcx*)B, ldb,
          0, mk(0.0, 0.0), false, (dcx*)W, M, M * N, mA_, mB_, kw, mt * kw, nt * kw, kchunk);
      splitk_reduce_kernel<dcx><<<rb, 256, 0, ctx->stream>>>(
          M, N, nsplit, (const dcx*)W, mk(beta.re, beta.im), use_beta, (dcx*)C, ldc);
    } else {
      gemm_simt_kernel<double><<<gs, 256, 0, ctx->stream>>>(
          opA, opB, M, N, K, alpha.re, (const double*)A, lda, 0, (const double*)B, ldb, 0, 0.0,
          false, (double*)W, M, M * N, mA_, mB_, kw, mt * kw, nt * kw, kchunk);
      splitk_reduce_kernel<double><<<rb, 256, 0, ctx->stream>>>(
          M, N, nsplit, (const double*)W, beta.re, use_beta, (double*)C, ldc);
    }
    LAUNCH_CHECK();
    count_launch_n(ctx, 2);
  } else if (is_cplx(dtype)) {
    gemm_simt_kernel<dcx><<<grid, 256, 0, ctx->stream>>>(
        opA, opB, M, N, K, mk(alpha.re, alpha.im), (const dcx*)A, lda, sA, (const dcx*)B, ldb,
        sB, mk(beta.re, beta.im), use_beta, (dcx*)C, ldc, sC, mA_, mB_, kw, mt * kw, nt * kw, 0);
    LAUNCH_CHECK();
    count_launch(ctx);
  } else {
    gemm_simt_kernel<double><<<grid, 256, 0, ctx->stream>>>(
        opA, opB, M, N, K, alpha.re, (const double*)A, lda, sA, (const double*)B, ldb, sB,
        beta.re, use_beta, (double*)C, ldc, sC, mA_, mB_, kw, mt * kw, nt * kw, 0);
    LAUNCH_CHECK();
    count_launch(ctx);
  }
  if (masks) GB_CHECK_CUDA(cudaFreeAsync(masks, ctx->stream));
}

// Same SIMT GEMM launched on a caller-provided stream, without a context (no scratch,
// no allocation, no launch counter); used by the allocation-free entry point.
cudaError_t gemm_fp64_on_stream(cudaStream_t stream, int dtype, char opA, char opB, int64_t M,
                                int64_t N, int64_t K, cplx alpha, const void* A, int64_t lda,
                                const void* B, int64_t ldb, cplx beta, void* C, int64_t ldc) {
  if (M == 0 || N == 0) return cudaSuccess;
  if ((N + GBN - 1) / GBN > 65535 || K <= 0) return cudaErrorInvalidValue;
  dim3 grid((unsigned)((M + GBM - 1) / GBM), (unsigned)((N + GBN - 1) / GBN), 1);
  bool use_beta = (beta.re != 0.0 || beta.im != 0.0);
  if (is_cplx(dtype)) {
    gemm_simt_kernel<dcx><<<grid, 256, 0, stream>>>(
        opA, opB, M, N, K, mk(alpha.re, alpha.im), (const dcx*)A, lda, 0, (const dcx*)B, ldb, 0,
        mk(beta.re, beta.im), use_beta, (dcx*)C, ldc, 0, nullptr, nullptr, 0, 0, 0, 0);
  } else {
    gemm_simt_kernel<double><<<grid, 256, 0, stream>>>(opA, opB, M, N, K, alpha.re,
                                                       (const double*)A, lda, 0, (const double*)B,
                                                       ldb, 0, beta.re, use_beta, (double*)C, ldc, 0,
                                                       nullptr, nullptr, 0, 0, 0, 0);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ BLAS-1
void fill_zero(gb_ctx* ctx, void* p, size_t bytes) {
  if (bytes == 0) return;
  GB_CHECK_CUDA(cudaMemsetAsync(p, 0, bytes, ctx->stream));
}

template <typename T>
__global__ void axpy_kernel(int64_t n, T a, const T* __restrict__ x, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = Ops<T>::fmaop(a, x[i], y[i]);
}
template <typename T>
__global__ void scale_kernel(int64_t n, T a, T* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = Ops<T>::mul(a, x[i]);
}

void axpy(gb_ctx* ctx, int dtype, int64_t n, cplx a, const void* x, void* y) {
  if (n == 0) return;
  unsigned nb = nblocks(n, 256, 152 * 16);
  if (is_cplx(dtype))
    axpy_kernel<dcx><<<nb, 256, 0, ctx->stream>>>(n, mk(a.re, a.im), (const dcx*)x, (dcx*)y);
  else
    axpy_kernel<double><<<nb, 256, 0, ctx->stream>>>(n, a.re, (const double*)x, (double*)y);
  LAUNCH_CHECK();
  count_launch(ctx);
}

void scale(gb_ctx* ctx, int dtype, int64_t n, cplx a, void* x) {
  if (n == 0) return;
  if (a.re == 0.0 && a.im == 0.0) {
    // scaling by zero writes zeros (VectorInterface.zerovector!): the contents of a fresh
    // allocation, NaN bit patterns included, do not survive
    GB_CHECK_CUDA(cudaMemsetAsync(x, 0, (size_t)n * elem_size(dtype), ctx->stream));
    return;
  }
  unsigned nb = nblocks(n, 256, 152 * 16);
  if (is_cplx(dtype))
    scale_kernel<dcx><<<nb, 256, 0, ctx->stream>>>(n, mk(a.re, a.im), (dcx*)x);
  else
    scale_kernel<double><<<nb, 256, 0, ctx->stream>>>(n, a.re, (double*)x);
  LAUNCH_CHECK();
  count_launch(ctx);
}

// Block reduction of two doubles with warp shuffles.
__device__ inline void block_reduce2(double& a, double& b) {
  __shared__ double sa[32], sb[32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) {
    sa[w] = a;
    sb[w] = b;
  }
  __syncthreads();
  int nw = blockDim.x / 32;
  if (w == 0) {
    a = l < nw ? sa[l] : 0.0;
    b = l < nw ? sb[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
}

constexpr int RED_BLOCKS = 152 * 4;

// partial[k * nblk + blk] = sum over this block's rows of conj(V[:,k]) . w  for k in [k0, k0+KC)
template <bool CPLX, int KC>
__global__ void __launch_bounds__(256)
    multidot_kernel(int64_t n, int k0, int k, const double* __restrict__ V, int64_t ld,
                    const double* __restrict__ w, double* __restrict__ part) {
  double re[KC], im[KC];
#pragma unroll
  for (int j = 0; j < KC; ++j) re[j] = im[j] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (CPLX) {
      double wr = w[2 * i], wi = w[2 * i + 1];
#pragma unroll
      for (int j = 0; j < KC; ++j) {
        if (k0 + j < k) {
          const double* v = V + 2 * (i + ld * (k0 + j));
          double vr = v[0], vi = v[1];
          re[j] = fma(vr, wr, fma(vi, wi, re[j]));
          im[j] = fma(vr, wi, fma(-vi, wr, im[j]));
        }
      }
    } else {
      double wr = w[i];
#pragma unroll
      for (int j = 0; j < KC; ++j)
        if (k0 + j < k) re[j] = fma(V[i + ld * (k0 + j)], wr, re[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < KC; ++j) {
    double a = re[j], b = im[j];
    block_reduce2(a, b);
    if (threadIdx.x == 0 && k0 + j < k) {
      part[2 * ((k0 + j) * (int64_t)gridDim.x + blockIdx.x)] = a;
      part[2 * ((k0 + j) * (int64_t)gridDim.x + blockIdx.x) + 1] = b;
    }
  }
}

__global__ void finish_reduce_kernel(int nblk, const double* __restrict__ part,
                                     double* __restrict__ out) {
  // one block per output value
  int j = blockIdx.x;
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += part[2 * ((int64_t)j * nblk + i)];
    b += part[2 * ((int64_t)j * nblk + i) + 1];
  }
  block_reduce2(a, b);
  if (threadIdx.x == 0) {
    out[2 * j] = a;
    out[2 * j + 1] = b;
  }
}

void multi_dot(gb_ctx* ctx, int dtype, int64_t n, int k, const void* V, int64_t ld,
               const void* w, cplx* host_out) {
  if (k == 0) return;
  int nblk = (int)std::min<int64_t>(RED_BLOCKS, std::max<int64_t>(1, (n + 255) / 256));
  size_t pb = sizeof(double) * 2 * ((size_t)k * nblk + k) + 256;
  double* part = (double*)scratch(ctx, SLOT_RED, pb);
  double* out = part + 2 * (size_t)k * nblk;
  constexpr int KC = 8;
  for (int k0 = 0; k0 < k; k0 += KC) {
    if (is_cplx(dtype))
      multidot_kernel<true, KC><<<nblk, 256, 0, ctx->stream>>>(n, k0, k, (const double*)V, ld,
                                                               (const double*)w, part);
    else
      multidot_kernel<false, KC><<<nblk, 256, 0, ctx->stream>>>(n, k0, k, (const double*)V, ld,
                                                                (const double*)w, part);
    LAUNCH_CHECK();
    count_launch(ctx);
  }
  finish_reduce_kernel<<<k, 256, 0, ctx->stream>>>(nblk, part, out);
  LAUNCH_CHECK();
  count_launch(ctx);
  if (ctx->h_pinned_elems < (size_t)2 * k) {
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    ctx->h_pinned_elems = std::max<size_t>(2 * k, 256);
    GB_CHECK_CUDA(cudaMallocHost(&ctx->h_pinned, sizeof(double) * ctx->h_pinned_elems));
  }
  GB_CHECK_CUDA(cudaMemcpyAsync(ctx->h_pinned, out, sizeof(double) * 2 * k,
                                cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int j = 0; j < k; ++j) host_out[j] = cplx{ctx->h_pinned[2 * j], ctx->h_pinned[2 * j + 1]};
}

cplx dot(gb_ctx* ctx, int dtype, int64_t n, const void* x, const void* y) {
  cplx r{0, 0};
  multi_dot(ctx, dtype, n, 1, x, n, y, &r);
  return r;
}

double nrm2(gb_ctx* ctx, int dtype, int64_t n, const void* x) {
  cplx r = dot(ctx, dtype, n, x, x);
  return std::sqrt(std::max(r.re, 0.0));
}

struct CoefPack {
  double c[2 * 64];
};

template <bool CPLX>
__global__ void multiaxpy_kernel(int64_t n, int k, const double* __restrict__ V, int64_t ld,
                                 CoefPack cf, double* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (CPLX) {
      double ar = w[2 * i], ai = w[2 * i + 1];
      for (int j = 0; j < k; ++j) {
        const double* v = V + 2 * (i + ld * j);
        double vr = v[0], vi = v[1], cr = cf.c[2 * j], ci = cf.c[2 * j + 1];
        ar = fma(vr, cr, fma(-vi, ci, ar));
        ai = fma(vr, ci, fma(vi, cr, ai));
      }
      w[2 * i] = ar;
      w[2 * i + 1] = ai;
    } else {
      double a = w[i];
      for (int j = 0; j < k; ++j) a = fma(V[i + ld * j], cf.c[2 * j], a);
      w[i] = a;
    }
  }
}

void multi_axpy(gb_ctx* ctx, int dtype, int64_t n, int k, const void* V, int64_t ld,
                const cplx* coef, void* w) {
  for (int j0 = 0; j0 < k; j0 += 64) {
    int kk = std::min(64, k - j0);
    CoefPack cf;
    for (int j = 0; j < kk; ++j) {
      cf.c[2 * j] = coef[j0 + j].re;
      cf.c[2 * j + 1] = coef[j0 + j].im;
    }
    unsigned nb = nblocks(n, 256, 152 * 16);
    const char* Vb = (const char*)V + (size_t)j0 * ld * elem_size(dtype);
    if (is_cplx(dtype))
      multiaxpy_kernel<true><<<nb, 256, 0, ctx->stream>>>(n, kk, (const double*)Vb, ld, cf,
                                                          (double*)w);
    else
      multiaxpy_kernel<false><<<nb, 256, 0, ctx->stream>>>(n, kk, (const double*)Vb, ld, cf,
                                                           (double*)w);
    LAUNCH_CHECK();
    count_launch(ctx);
  }
}

__global__ void finite_kernel(int64_t n, const double* __restrict__ x, int* flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(x[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

bool all_finite(gb_ctx* ctx, int dtype, int64_t n, const void* x) {
  int* flag = (int*)scratch(ctx, SLOT_TMP2, 256);
  GB_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
  int64_t nd = n * (is_cplx(dtype) ? 2 : 1);
  finite_kernel<<<nblocks(nd, 256, 152 * 8), 256, 0, ctx->stream>>>(nd, (const double*)x, flag);
  LAUNCH_CHECK();
  count_launch(ctx);
  int h = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return h == 0;
}

}  // namespace gb
