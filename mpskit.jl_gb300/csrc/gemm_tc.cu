// Split-precision GEMM on the 5th-generation tensor cores (sm_103a).
//
// Scheme ("bf16x3", a published split-operand scheme; see e.g. Henry, Tang & Heinecke,
// "Leveraging the bfloat16 Artificial Intelligence Datatype For Higher-Precision
// Computations", ARITH 2019): every FP64 operand x is split into hi = bf16(x) and
// lo = bf16(x - hi); the product is hi*hi + hi*lo + lo*hi accumulated in FP32.  The
// three products are one K-loop over (pair, k-block) that re-reads the hi/lo planes.
// "tf32x3" is the same scheme with TF32 planes (hi = tf32(x), lo = tf32(x - hi), each held
// in a 32-bit word, tcgen05 kind::tf32): 22 significant bits per operand instead of 16.
//
// Complex operands are realified: A' = [Re A | Im A] along K and
// B' = [[Re B; -Im B] | [Im B; Re B]] along N, so C' = A' B'^T = [Re C | Im C].
//
// Kernel: one CTA per 128 x 256 output tile; warp 0 issues TMA loads (128B swizzle) into
// a 4-stage shared-memory ring guarded by mbarriers, warp 1 owns the TMEM accumulator
// (tcgen05.alloc) and issues tcgen05.mma (M=128, N=256, K=16, BF16 -> FP32) from one
// thread, warps 2-5 drain TMEM with tcgen05.ld and write FP64 C = alpha*acc + beta*C.
// Every mbarrier wait is bounded in time; on expiry the kernel records GB_ERR_TIMEOUT in
// the context status word, drains its outstanding copies and frees TMEM before exiting.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "gb_common.h"
#include "tc_ptx.cuh"

namespace gb {

constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
constexpr int TC_BK = 64;  // bf16 elements per 128-byte row
constexpr int TC_STAGES = 4;
constexpr int TC_THREADS = 192;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr int TC_SMEM_BYTES = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int64_t KALIGN = TC_BK;

static inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// ------------------------------------------------------------------ packing
// out layout: [batch][plane(2)][rows][Kp] bf16 ; rows = M (A) or N / 2N (B, complex)
struct PackArgs {
  int role;      // 0 = A (rows = M), 1 = B (rows = N)
  char op;
  int cplx;
  int64_t R;     // logical rows (M for A, N for B)
  int64_t K;     // logical K
  int64_t Kh;    // imaginary-half offset along K (complex)
  int64_t Kp;    // padded packed K
  int64_t rows;  // packed rows (R, or 2R for complex B)
  int64_t ld, stride;
};

// element (r, k) of the logical operand: A -> op(A)[r, k], B -> op(B)[k, r]
__device__ inline void load_elem(const PackArgs& p, const double* src, int64_t r, int64_t k,
                                 double& re, double& im) {
  int64_t addr;
  bool rowfast;  // r is the leading (contiguous) index of the source
  if (p.role == 0) rowfast = (p.op == 'N');
  else rowfast = (p.op != 'N');
  addr = rowfast ? (r + p.ld * k) : (k + p.ld * r);
  if (p.cplx) {
    re = src[2 * addr];
    im = src[2 * addr + 1];
    if (p.op == 'C') im = -im;
  } else {
    re = src[addr];
    im = 0.0;
  }
}

// 32 x 32 tile transpose through shared memory; block = 32 x 8 threads.
template <typename E>
__global__ void pack_kernel(PackArgs p, const double* __restrict__ src, E* __restrict__ dst,
                            uint32_t* __restrict__ mask, int kw, int64_t mrows) {
  __shared__ double tre[32][33];
  __shared__ double tim[32][33];
  const int64_t b = blockIdx.z;
  src += b * p.stride * (p.cplx ? 2 : 1);
  E* hi = dst + b * 2 * p.rows * p.Kp;
  E* lo = hi + p.rows * p.Kp;
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  bool rowfast = (p.role == 0) ? (p.op == 'N') : (p.op != 'N');
  // load: contiguous source index on threadIdx.x
  for (int j = ty; j < 32; j += 8) {
    int64_t r, k;
    if (rowfast) {
      r = r0 + tx;
      k = k0 + j;
    } else {
      k = k0 + tx;
      r = r0 + j;
    }
    double re = 0.0, im = 0.0;
    if (r < p.R && k < p.K) load_elem(p, src, r, k, re, im);
    int rr = (int)(r - r0), kk = (int)(k - k0);
    tre[rr][kk] = re;
    tim[rr][kk] = im;
  }
  __syncthreads();
  // store: k fastest
  int nz = 0;
  for (int j = ty; j < 32; j += 8) {
    int64_t r = r0 + j, k = k0 + tx;
    if (r >= p.R || k >= p.Kh) continue;  // entries k >= K were loaded as zeros
    double re = tre[j][tx], im = tim[j][tx];
    nz |= (re != 0.0 || im != 0.0);
    auto put = [&](int64_t row, int64_t col, double v) {
      split_put_f(hi, lo, row * p.Kp + col, (float)v);
    };
    if (!p.cplx) {
      put(r, k, re);
    } else if (p.role == 0) {
      put(r, k, re);
      put(r, p.Kh + k, im);
    } else {
      put(r, k, re);
      put(r, p.Kh + k, -im);
      put(p.R + r, k, im);
      put(p.R + r, p.Kh + k, re);
    }
  }
  // nonzero map: this 32 x 32 block lies in one 128-row tile and one k-block
  // (complex operands also touch the imaginary half; marked conservatively)
  if (__syncthreads_or(nz) && tx == 0 && ty == 0) {
    uint32_t* mb = mask + b * mrows * kw;
    auto mark = [&](int64_t row, int64_t col) {
      int64_t kb = col / bk_of<E>();
      atomicOr(&mb[(row / MASK_ROWS) * kw + kb / 32], 1u << (kb % 32));
    };
    const int64_t rlast = std::min<int64_t>(r0 + 31, p.R - 1);
    mark(r0, k0);
    if (p.cplx) {
      mark(r0, p.Kh + k0);
      if (p.role == 1) {
        mark(p.R + r0, k0);
        mark(p.R + r0, p.Kh + k0);
        mark(p.R + rlast, k0);
        mark(p.R + rlast, p.Kh + k0);
      }
    }
  }
}

static size_t plane_bytes(int64_t prow, int64_t Kp, int64_t batch, int esz) {
  return (size_t)round_up((int64_t)batch * 2 * prow * Kp * esz, 256);
}
static int mask_words(int64_t Kp, int bk) { return (int)((Kp / bk + 31) / 32); }

size_t packed_bytes(int64_t rows, int64_t K, bool cplx, int role, int64_t batch, int prec) {
  const int esz = is_tf32(prec) ? 4 : 2, bk = 128 / esz;
  int64_t Kh = round_up(std::max<int64_t>(K, 1), KALIGN);
  int64_t Kp = cplx ? 2 * Kh : Kh;
  int64_t prow = (cplx && role == PACK_AS_B) ? 2 * rows : rows;
  int64_t mrows = (prow + MASK_ROWS - 1) / MASK_ROWS;
  return plane_bytes(prow, Kp, batch, esz) + (size_t)batch * mrows * mask_words(Kp, bk) * 4 +
         (size_t)batch * Kp * 4;
}

void packed_layout(Packed& out, void* data, int64_t R, int64_t K, bool cx, int role,
                   int64_t batch, int prec) {
  out.esz = is_tf32(prec) ? 4 : 2;
  out.bk = 128 / out.esz;
  out.data = data;
  out.K = K;
  out.Kh = round_up(std::max<int64_t>(K, 1), KALIGN);
  out.Kp = cx ? 2 * out.Kh : out.Kh;
  out.rows = (cx && role == PACK_AS_B) ? 2 * R : R;
  out.batch = batch;
  out.cplx = cx;
  out.bytes = packed_bytes(R, K, cx, role, batch, prec);
  out.mrows = (out.rows + MASK_ROWS - 1) / MASK_ROWS;
  out.kw = mask_words(out.Kp, out.bk);
  out.mask = (uint32_t*)((char*)data + plane_bytes(out.rows, out.Kp, batch, out.esz));
  out.cnt = out.mask + (size_t)batch * out.mrows * out.kw;
  out.cnt_valid = false;
}

// nonzero rows per packed k (both planes), rows split in chunks of 256 with one atomic each
template <typename E>
__global__ void count_cols_kernel(const E* __restrict__ planes, int64_t rows, int64_t Kp,
                                  uint32_t* __restrict__ cnt) {
  const int64_t b = blockIdx.z;
  const E* hi = planes + b * 2 * rows * Kp;
  const E* lo = hi + rows * Kp;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= Kp) return;
  const int64_t r0 = (int64_t)blockIdx.y * 256, r1 = std::min<int64_t>(r0 + 256, rows);
  uint32_t c = 0;
  for (int64_t r = r0; r < r1; ++r)
    c += (plane_nz(hi[r * Kp + k]) || plane_nz(lo[r * Kp + k]));
  if (c) atomicAdd(&cnt[b * Kp + k], c);
}

static void count_cols(gb_ctx* ctx, Packed& p) {
  GB_CHECK_CUDA(cudaMemsetAsync(p.cnt, 0, (size_t)p.batch * p.Kp * 4, ctx->stream));
  dim3 grid((unsigned)((p.Kp + 255) / 256), (unsigned)((p.rows + 255) / 256), (unsigned)p.batch);
  GB_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "count: grid too large");
  if (p.esz == 4)
    count_cols_kernel<float><<<grid, 256, 0, ctx->stream>>>((const float*)p.data, p.rows, p.Kp,
                                                            p.cnt);
  else
    count_cols_kernel<__nv_bfloat16><<<grid, 256, 0, ctx->stream>>>(
        (const __nv_bfloat16*)p.data, p.rows, p.Kp, p.cnt);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  p.cnt_valid = true;
}

// work[1] += 2 sum_z sum_k cntA[z][k] cntB[z][k]
__global__ void nonzero_products_kernel(const uint32_t* __restrict__ ca, const uint32_t* __restrict__ cb,
                                        int64_t Kp, int64_t batch, int sa, int sb,
                                        double* __restrict__ work) {
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < Kp * batch;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = e / Kp, k = e % Kp;
    acc += (double)ca[(sa ? z : 0) * Kp + k] * (double)cb[(sb ? z : 0) * Kp + k];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(&work[1], 2.0 * acc);
}

static void clear_mask(gb_ctx* ctx, const Packed& p) {
  GB_CHECK_CUDA(cudaMemsetAsync(p.mask, 0, (size_t)p.batch * p.mrows * p.kw * 4, ctx->stream));
}

void pack_operand(gb_ctx* ctx, int dtype, int role, char op, int64_t R, int64_t K,
                  const void* src, int64_t ld, int64_t stride, int64_t batch, Packed& out,
                  void* dst, int prec) {
  bool cx = is_cplx(dtype);
  PackArgs p;
  p.role = role;
  p.op = op;
  p.cplx = cx;
  p.R = R;
  p.K = K;
  p.Kh = round_up(std::max<int64_t>(K, 1), KALIGN);
  p.Kp = cx ? 2 * p.Kh : p.Kh;
  p.rows = (cx && role == PACK_AS_B) ? 2 * R : R;
  p.ld = ld;
  p.stride = stride;
  packed_layout(out, dst, R, K, cx, role, batch, prec);
  // the planes need no memset: the kernel writes every (row, k < Kh) entry, zeros
  // included for k >= K; only the nonzero map starts cleared
  clear_mask(ctx, out);
  GB_REQUIRE(batch <= 65535 && (R + 31) / 32 <= 65535, "pack: grid too large");
  dim3 grid((unsigned)((p.Kh + 31) / 32), (unsigned)((R + 31) / 32), (unsigned)batch);
  if (out.esz == 4)
    pack_kernel<float><<<grid, dim3(32, 8), 0, ctx->stream>>>(p, (const double*)src, (float*)dst,
                                                              out.mask, out.kw, out.mrows);
  else
    pack_kernel<__nv_bfloat16><<<grid, dim3(32, 8), 0, ctx->stream>>>(
        p, (const double*)src, (__nv_bfloat16*)dst, out.mask, out.kw, out.mrows);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  if (ctx->counting) count_cols(ctx, out);
}

// ------------------------------------------------------------------ fused leg mix + pack
// y[a + out_off[J] + n*yn] = sum_e val[e] x[a + in_off[col[e]] + n*xn] written directly as
// the packed B operand of the following GEMM: logical B element (k, m) with
// k = a + kJ[J] (contraction index) and m = mJ[J] + n*mn (output column index).
template <bool CPLX, typename E, typename TX>
__global__ void mixpack_kernel(int64_t A, int64_t N, int64_t xn, const int64_t* __restrict__ in_off,
                               const int64_t* __restrict__ kJ, const int64_t* __restrict__ mJ,
                               int64_t mn, const int* __restrict__ row_ptr,
                               const int* __restrict__ col, const double* __restrict__ val,
                               const TX* __restrict__ x, E* __restrict__ hi, int64_t Nlog,
                               int64_t Kp, int64_t Kh, int64_t plane, uint32_t* __restrict__ mask,
                               int kw, MixSkipDev sk) {
  constexpr int BK = bk_of<E>();
  const int J = blockIdx.y;
  const int e0 = row_ptr[J], e1 = row_ptr[J + 1];
  const int lane = threadIdx.x % 32;
  E* lo = hi + plane;
  auto put = [&](int64_t row, int64_t c, double v) { split_put_f(hi, lo, row * Kp + c, (float)v); };
  auto mark = [&](int64_t row, int64_t kb) {
    atomicOr(&mask[(row / MASK_ROWS) * kw + kb / 32], 1u << (kb % 32));
  };
  for (int64_t n = blockIdx.z; n < N; n += gridDim.z) {
    const int64_t m = mJ[J] + n * mn;
    // U(1): only the l' sector of (J, n) can be nonzero; every entry of it is written on
    // every call, and the rest of the operand stays zero from its allocation
    int64_t lo = 0, hi = A;
    if (sk.arange) {
      const int2 r = sk.arange[n * gridDim.y + J];
      lo = r.x;
      hi = r.y;
    }
    // every thread of the block runs the same number of iterations (warp-wide votes below)
    for (int64_t base = lo + blockIdx.x * (int64_t)blockDim.x; base < hi;
         base += (int64_t)gridDim.x * blockDim.x) {
      const int64_t a = base + threadIdx.x;
      bool valid = a < hi;
      const int64_t k = a + kJ[J];
      bool nz = false;
      // input e of element (a, n) lies in box (row, column) of x's written-region map; the
      // producer keeps every region outside the map at zero
      auto box_set = [&](int i, int64_t row) {
        const int64_t bit = ((row + sk.roff[i]) >> 7) * sk.onc + ((sk.coff[i] + n * sk.xnM) >> 7);
        return ((sk.xmap[bit >> 5] >> (bit & 31)) & 1u) != 0u;
      };
      if (sk.xmap && !sk.arange) {
        // warp-wide test first: the warp's 32 rows span at most two row boxes per input, so
        // one pass of the lanes over the inputs decides whether anything is there to read
        const int64_t wa0 = base + (threadIdx.x & ~31);
        const int64_t wa1 = (wa0 + 31 < A ? wa0 + 31 : A - 1);
        bool hit = false;
        if (wa0 < A)
          for (int e = e0 + lane; e < e1 && !hit; e += 32) {
            const int i = col[e];
            hit = box_set(i, wa0) || box_set(i, wa1);
          }
        hit = __any_sync(0xffffffffu, hit);
        if (!hit) {
          // nothing to read: the output is zero; it is written only where the previous
          // apply marked its box (the planes hold zeros everywhere else)
          if (valid) {
            const int64_t kb0 = k / BK;
            auto prev = [&](int64_t row, int64_t kb) {
              return (sk.prev[(row / MASK_ROWS) * kw + kb / 32] >> (kb % 32)) & 1u;
            };
            if (prev(m, kb0)) put(m, k, 0.0);
            if (CPLX) {
              if (prev(m, kb0 + Kh / BK)) put(m, Kh + k, 0.0);
              if (prev(Nlog + m, kb0)) put(Nlog + m, k, 0.0);
              if (prev(Nlog + m, kb0 + Kh / BK)) put(Nlog + m, Kh + k, 0.0);
            }
          }
          valid = false;  // nothing to compute or mark
        }
      }
      if (valid) {
        if (CPLX) {
          double re = 0.0, im = 0.0;
          for (int e = e0; e < e1; ++e) {
            const TX* xv = x + 2 * (a + in_off[col[e]] + n * xn);
            const double xr = xv[0], xi = xv[1];
            double vr = val[2 * e], vi = val[2 * e + 1];
            re = fma(vr, xr, fma(-vi, xi, re));
            im = fma(vr, xi, fma(vi, xr, im));
          }
          put(m, k, re);
          put(m, Kh + k, -im);
          put(Nlog + m, k, im);
          put(Nlog + m, Kh + k, re);
          nz = (re != 0.0 || im != 0.0);
        } else {
          double acc = 0.0;
          for (int e = e0; e < e1; ++e)
            acc = fma(val[e], (double)x[a + in_off[col[e]] + n * xn], acc);
          put(m, k, acc);
          nz = acc != 0.0;
        }
      }
      // one atomic per (k-block, warp): the first lane with a nonzero value in its group
      const int64_t kb = valid ? k / BK : -1;
      const unsigned grp = __match_any_sync(0xffffffffu, kb);
      const unsigned nzb = __ballot_sync(0xffffffffu, nz);
      if (nz && lane == __ffs(grp & nzb) - 1) {
        mark(m, kb);
        if (CPLX) {
          mark(m, kb + Kh / BK);
          mark(Nlog + m, kb);
          mark(Nlog + m, kb + Kh / BK);
        }
      }
    }
  }
}

void mixpack_run(gb_ctx* ctx, const MixDev& m, const int64_t* kJ, const int64_t* mJ, int64_t mn,
                 int dtype, const void* x, Packed& out, int64_t Klog, int64_t Nlog,
                 const MixSkipDev* skip, bool x_f32) {
  const bool cx = is_cplx(dtype);
  GB_REQUIRE(m.nJ <= 65535, "mixpack: too many output rows");
  GB_REQUIRE(m.xa == 1, "mixpack: unit input stride required");
  // zero the K padding of every row (entries k >= Klog are never produced by the mix); with
  // skipping, the planes were zeroed at allocation and the padding is never written
  if (out.Kh > Klog && !(skip && skip->xmap)) {
    const int64_t es = out.esz;
    const int64_t planes = 2 * out.batch;
    for (int64_t p = 0; p < planes; ++p) {
      char* pb = (char*)out.data + p * out.rows * out.Kp * es;
      GB_CHECK_CUDA(cudaMemset2DAsync(pb + Klog * es, out.Kp * es, 0, (out.Kh - Klog) * es,
                                      out.rows, ctx->stream));
      if (cx)
        GB_CHECK_CUDA(cudaMemset2DAsync(pb + (out.Kh + Klog) * es, out.Kp * es, 0,
                                        (out.Kh - Klog) * es, out.rows, ctx->stream));
    }
  }
  GB_REQUIRE(out.batch == 1 && out.mask, "mixpack: single packed operand with a map");
  MixSkipDev sk{};
  if (skip && skip->xmap) {
    // the planes were zeroed at allocation and entries are skipped only where they are
    // known zero: keep the previous map to know which boxes may hold stale nonzeros
    sk = *skip;
    GB_CHECK_CUDA(cudaMemcpyAsync(sk.prev, out.mask, (size_t)out.mrows * out.kw * 4,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  }
  clear_mask(ctx, out);
  // a block walks N / gridDim.z output columns: long-lived blocks, since with structural
  // skipping most of a block's work is a map test
  const int64_t span = sk.arange ? std::max<int64_t>(sk.arange_max, 1) : m.A;
  dim3 grid((unsigned)std::min<int64_t>((span + 127) / 128, 64), (unsigned)m.nJ,
            (unsigned)std::min<int64_t>(m.N, 32));
  const int64_t plane = out.rows * out.Kp;
#define GB_MIXPACK(C, E, TX)                                                                  \
  mixpack_kernel<C, E, TX><<<grid, 128, 0, ctx->stream>>>(                                    \
      m.A, m.N, m.xn, m.in_off, kJ, mJ, mn, m.row_ptr, m.col, m.val, (const TX*)x,            \
      (E*)out.data, Nlog, out.Kp, out.Kh, plane, out.mask, out.kw, sk)
#define GB_MIXPACK_X(C, E)          \
  do {                              \
    if (x_f32) GB_MIXPACK(C, E, float); \
    else GB_MIXPACK(C, E, double);  \
  } while (0)
  if (out.esz == 4) {
    if (cx) GB_MIXPACK_X(true, float);
    else GB_MIXPACK_X(false, float);
  } else {
    if (cx) GB_MIXPACK_X(true, __nv_bfloat16);
    else GB_MIXPACK_X(false, __nv_bfloat16);
  }
#undef GB_MIXPACK_X
#undef GB_MIXPACK
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  out.cnt_valid = false;
  if (ctx->counting) count_cols(ctx, out);
}


struct TcArgs {
  int64_t M, N;        // logical output (N = packed B rows, i.e. 2N when complex)
  int64_t Nlog;        // logical N (complex: real/imag split point)
  int cplx;
  int kblocks;         // Kp / 64
  int batchA, batchB;  // 1 when the operand is shared across the batch
  double alpha, beta;
  double* C;
  int64_t ldc, sC;
  int* status;
  unsigned long long wait_ns;  // bound on every pipeline wait (drains use DRAIN_WAIT_NS)
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap mapA,
                       const __grid_constant__ CUtensorMap mapB, TcArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* full = bars;                    // [TC_STAGES]
  uint64_t* empty = bars + TC_STAGES;       // [TC_STAGES]
  uint64_t* accum = bars + 2 * TC_STAGES;   // [1]
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * TC_STAGES + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int64_t m0 = (int64_t)blockIdx.x * TC_BM;
  const int64_t n0 = (int64_t)blockIdx.y * TC_BN;
  const int bz = blockIdx.z;
  const int total = 3 * args.kblocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(accum), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    bool ok = true;
    for (int it = 0; it < total && ok; ++it) {
      int s = it % TC_STAGES;
      uint32_t round = it / TC_STAGES;
      ok = mbar_wait_bounded(smem_u32(&empty[s]), (round & 1) ^ 1, args.status, args.wait_ns);
      if (!ok) break;
      int pair = it / args.kblocks, kb = it % args.kblocks;
      int planeA = (pair == 2) ? 1 : 0, planeB = (pair == 1) ? 1 : 0;
      uint32_t sa = smem_u32(smem + s * TC_STAGE_BYTES);
      uint32_t sb = sa + TC_A_BYTES;
      uint32_t fb = smem_u32(&full[s]);
      mbar_expect_tx(fb, TC_STAGE_BYTES);
      int za = (args.batchA > 1 ? bz : 0) * 2 + planeA;
      int zb = (args.batchB > 1 ? bz : 0) * 2 + planeB;
      tma_load_3d(sa, &mapA, fb, kb * TC_BK, (int)m0, za);
      tma_load_3d(sb, &mapB, fb, kb * TC_BK, (int)n0, zb);
      ++issued;
    }
    if (!ok) {
      // drain copies still in flight before this CTA may exit
      for (int it = std::max(0, issued - TC_STAGES); it < issued; ++it) {
        int s = it % TC_STAGES;
        mbar_wait_bounded(smem_u32(&full[s]), (it / TC_STAGES) & 1, args.status, DRAIN_WAIT_NS);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    const uint32_t idesc = idesc_bf16(TC_BM, TC_BN);
    bool ok = true;
    for (int it = 0; it < total; ++it) {
      int s = it % TC_STAGES;
      ok = mbar_wait_bounded(smem_u32(&full[s]), (it / TC_STAGES) & 1, args.status, args.wait_ns);
      if (!ok) break;
      tc_fence_after();
      uint32_t sa = smem_u32(smem + s * TC_STAGE_BYTES);
      uint32_t sb = sa + TC_A_BYTES;
      uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sb);
#pragma unroll
      for (int k = 0; k < TC_BK / 16; ++k) {
        // advance 16 bf16 = 32 bytes inside the 128-byte swizzle atom
        mma_bf16(tmem, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), idesc,
                 (it > 0 || k > 0) ? 1u : 0u);
      }
      mma_commit(smem_u32(&empty[s]));
    }
    mma_commit(smem_u32(accum));
    // every MMA issued by this thread has retired before TMEM is released
    mbar_wait_bounded(smem_u32(accum), 0, args.status, DRAIN_WAIT_NS);
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> FP64 global
    const int g = warp % 4;  // TMEM lane quarter accessible by this warp
    bool ok = mbar_wait_bounded(smem_u32(accum), 0, args.status, args.wait_ns);
    tc_fence_after();
    const int64_t m = m0 + 32 * g + lane;
    double* C = args.C + (int64_t)bz * args.sC * (args.cplx ? 2 : 1);
#pragma unroll 1
    for (int c0 = 0; c0 < TC_BN; c0 += 32) {
      uint32_t r[32];
      uint32_t taddr = tmem + ((uint32_t)(32 * g) << 16) + (uint32_t)c0;
      TMEM_LD32(taddr, r);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (!ok || m >= args.M) continue;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        int64_t n = n0 + c0 + j;
        if (n >= args.N) break;
        double v = (double)__uint_as_float(r[j]);
        if (args.alpha != 1.0) v *= args.alpha;
        double* p;
        if (args.cplx) {
          int64_t nn = n < args.Nlog ? n : n - args.Nlog;
          p = C + 2 * (m + args.ldc * nn) + (n < args.Nlog ? 0 : 1);
        } else {
          p = C + m + args.ldc * n;
        }
        if (args.beta != 0.0) v = fma(args.beta, *p, v);
        *p = v;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_BN));
  }
}

// ------------------------------------------------------------------ persistent kernel
// One CTA per SM walks output tiles handed out by a global counter.  The producer warp
// fetches a tile, computes its k-block list (all k-blocks, or those whose A-tile and B-tile
// nonzero bits are both set) and publishes (tile, count) through a small ring in shared
// memory to the MMA warp and the four epilogue warps.  The accumulator is double-buffered
// in TMEM (2 x BN columns): the epilogue drains tile i while the MMAs of tile i+1 run.
struct PArgs {
  int64_t M, N, Nlog;  // N = packed B rows (2N when complex)
  int cplx;
  int kblocks;         // Kp / 64
  int mt, nt;          // output tiles along M (128) and N (BN)
  int ntiles;          // mt * nt * batch
  int batchA, batchB;
  double alpha, beta;
  double* C;
  int64_t ldc, sC;
  const uint32_t* maskA;  // null: every k-block
  const uint32_t* maskB;
  int kw;
  int64_t mskA_b, mskB_b;  // words per batch entry
  int64_t mrowsB;
  unsigned int* counter;
  int* status;
  unsigned long long wait_ns;  // bound on every pipeline wait (drains use DRAIN_WAIT_NS)
  double* work;  // when set: += tensor-pipe flops per split product of every tile
  // optional output map: bit (m / 128) * onc + (logical column / 128) is set for every
  // output tile that receives a contribution; with skip_zero_out, tiles that receive none
  // are not written at all (the consumer reads C only where the map is set)
  uint32_t* outmap;
  const uint32_t* prevmap;  // the previous call's map: its tiles are zeroed if not rewritten
  int64_t onc;
  int skip_zero_out;
  int c_f32;  // C is stored in FP32 (exact when alpha = 1 and beta = 0: C is the accumulator)
};

constexpr int PS_RING = 4;


template <int BN>
struct TileMasks {
  const uint32_t* a;
  const uint32_t* b;
  int nb;  // mask rows of B covered by this tile
  __device__ __forceinline__ uint32_t word(int w, int kw) const {
    uint32_t bw = 0;
    for (int q = 0; q < nb; ++q) bw |= b[q * kw + w];
    return a[w] & bw;
  }
};

template <int BN>
__device__ __forceinline__ TileMasks<BN> tile_masks(const PArgs& p, int mi, int ni, int z) {
  TileMasks<BN> t;
  t.a = p.maskA + (p.batchA > 1 ? z : 0) * p.mskA_b + (int64_t)mi * p.kw;
  int64_t r0 = (int64_t)ni * (BN / MASK_ROWS);
  t.b = p.maskB + (p.batchB > 1 ? z : 0) * p.mskB_b + r0 * p.kw;
  t.nb = (int)std::min<int64_t>(BN / MASK_ROWS, p.mrowsB - r0);
  return t;
}

template <int BN, int STAGES, bool TF32>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_bf16x3_persistent(const __grid_constant__ CUtensorMap mapA,
                           const __grid_constant__ CUtensorMap mapB, PArgs args) {
  constexpr int BKE = TF32 ? 32 : 64;  // k elements per stage (one 128-byte swizzle row)
  constexpr int A_BYTES = TC_BM * 128;
  constexpr int B_BYTES = BN * 128;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* full = bars;                        // [STAGES]  TMA -> MMA
  uint64_t* empty = full + STAGES;              // [STAGES]  MMA -> TMA
  uint64_t* tfull = empty + STAGES;             // [2]       MMA -> epilogue
  uint64_t* tempty = tfull + 2;                 // [2]       epilogue -> MMA
  uint64_t* sfull = tempty + 2;                 // [RING]    producer -> consumers
  uint64_t* sempty = sfull + PS_RING;           // [RING]    consumers -> producer
  uint64_t* done = sempty + PS_RING;            // [1]       all MMAs retired
  int* stile = (int*)(done + 1);                // [RING]
  int* snk = stile + PS_RING;                   // [RING]
  uint32_t* tmem_slot = (uint32_t*)(snk + PS_RING);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int mn = args.mt * args.nt;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);
    }
    for (int r = 0; r < PS_RING; ++r) {
      mbar_init(smem_u32(&sfull[r]), 1);
      mbar_init(smem_u32(&sempty[r]), 5);  // MMA thread + 4 epilogue warps
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- scheduler + TMA producer
    uint32_t g = 0, issued = 0;
    bool ok = true;
    for (int j = 0; ok; ++j) {
      int t = -1, nk = 0, mi = 0, ni = 0, z = 0;
      for (;;) {
        int c = (int)atomicAdd(args.counter, 1u);
        if (c >= args.ntiles) break;
        z = c / mn;
        int r = c - z * mn;
        ni = r / args.mt;
        mi = r - ni * args.mt;
        if (args.maskA) {
          TileMasks<BN> tm = tile_masks<BN>(args, mi, ni, z);
          nk = 0;
          for (int w = 0; w < args.kw; ++w) nk += __popc(tm.word(w, args.kw));
        } else {
          nk = args.kblocks;
        }
        if (nk > 0 || (args.beta != 1.0 && !args.skip_zero_out)) {
          t = c;
          break;
        }
        if (args.prevmap && args.beta == 0.0) {
          // written by the previous call, nothing this time: overwrite with zeros
          const int64_t n0 = (int64_t)ni * BN, n1 = std::min<int64_t>(n0 + BN, args.N);
          bool stale = false;
          for (int64_t g = n0 / 128; g <= (n1 - 1) / 128 && !stale; ++g) {
            const int64_t bit = (int64_t)mi * args.onc + g;
            stale = (args.prevmap[bit >> 5] >> (bit & 31)) & 1u;
          }
          if (stale) {
            t = c;
            break;
          }
        }
      }
      const int slot = j % PS_RING;
      ok = mbar_wait_bounded(smem_u32(&sempty[slot]), ((j / PS_RING) & 1) ^ 1, args.status, args.wait_ns);
      if (!ok) break;
      stile[slot] = t;
      snk[slot] = nk;
      mbar_arrive(smem_u32(&sfull[slot]));
      if (t < 0) break;
      if (nk == 0) continue;
      if (args.work) atomicAdd(args.work, (double)nk * (2.0 * TC_BM * BN * BKE));
      if (args.outmap) {
        // logical column groups of this tile (complex: real and imaginary halves)
        const int64_t n0 = (int64_t)ni * BN, n1 = std::min<int64_t>(n0 + BN, args.N);
        auto set_range = [&](int64_t c0, int64_t c1) {
          for (int64_t g = c0 / 128; g <= (c1 - 1) / 128; ++g) {
            const int64_t bit = (int64_t)mi * args.onc + g;
            atomicOr(&args.outmap[bit >> 5], 1u << (bit & 31));
          }
        };
        if (!args.cplx) {
          set_range(n0, n1);
        } else {
          if (n0 < args.Nlog) set_range(n0, std::min(n1, args.Nlog));
          if (n1 > args.Nlog) set_range(std::max(n0, args.Nlog) - args.Nlog, n1 - args.Nlog);
        }
      }
      const int64_t m0 = (int64_t)mi * TC_BM, n0 = (int64_t)ni * BN;
      const int za0 = (args.batchA > 1 ? z : 0) * 2, zb0 = (args.batchB > 1 ? z : 0) * 2;
      TileMasks<BN> tm;
      if (args.maskA) tm = tile_masks<BN>(args, mi, ni, z);
      for (int pair = 0; pair < 3 && ok; ++pair) {
        const int planeA = (pair == 2) ? 1 : 0, planeB = (pair == 1) ? 1 : 0;
        for (int w = 0; w < (args.maskA ? args.kw : 1) && ok; ++w) {
          uint32_t bits = args.maskA ? tm.word(w, args.kw) : 0u;
          int kb = args.maskA ? -1 : 0;
          for (;;) {
            if (args.maskA) {
              if (!bits) break;
              kb = w * 32 + __ffs(bits) - 1;
              bits &= bits - 1;
            } else if (kb >= args.kblocks) {
              break;
            }
            const int s = g % STAGES;
            ok = mbar_wait_bounded(smem_u32(&empty[s]), ((g / STAGES) & 1) ^ 1, args.status, args.wait_ns);
            if (!ok) break;
            const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
            const uint32_t fb = smem_u32(&full[s]);
            mbar_expect_tx(fb, STAGE_BYTES);
            tma_load_3d(sa, &mapA, fb, kb * BKE, (int)m0, za0 + planeA);
            tma_load_3d(sa + A_BYTES, &mapB, fb, kb * BKE, (int)n0, zb0 + planeB);
            ++g;
            ++issued;
            if (!args.maskA) ++kb;
          }
        }
      }
    }
    if (!ok) {
      // drain copies still in flight before this CTA may exit
      for (uint32_t it = issued > (uint32_t)STAGES ? issued - STAGES : 0; it < issued; ++it) {
        const int s = it % STAGES;
        mbar_wait_bounded(smem_u32(&full[s]), (it / STAGES) & 1, args.status, DRAIN_WAIT_NS);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    const uint32_t idesc = TF32 ? idesc_tf32(TC_BM, BN) : idesc_bf16(TC_BM, BN);
    uint32_t g = 0, acc = 0;
    bool ok = true;
    for (int j = 0; ok; ++j) {
      const int slot = j % PS_RING;
      ok = mbar_wait_bounded(smem_u32(&sfull[slot]), (j / PS_RING) & 1, args.status, args.wait_ns);
      if (!ok) break;
      const int t = stile[slot], nk = snk[slot];
      mbar_arrive(smem_u32(&sempty[slot]));
      if (t < 0) break;
      if (nk == 0) continue;
      const uint32_t buf = acc & 1;
      ok = mbar_wait_bounded(smem_u32(&tempty[buf]), ((acc >> 1) & 1) ^ 1, args.status, args.wait_ns);
      if (!ok) break;
      tc_fence_after();
      const uint32_t d = tmem + buf * BN;
      const int total = 3 * nk;
      for (int it = 0; it < total; ++it) {
        const int s = g % STAGES;
        ok = mbar_wait_bounded(smem_u32(&full[s]), (g / STAGES) & 1, args.status, args.wait_ns);
        if (!ok) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
        const uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sa + A_BYTES);
        // four MMAs of 32 bytes of K each (16 BF16 or 8 TF32): +2 in 16-byte units
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (TF32)
            mma_tf32(d, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), idesc,
                     (it > 0 || k > 0) ? 1u : 0u);
          else
            mma_bf16(d, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), idesc,
                     (it > 0 || k > 0) ? 1u : 0u);
        }
        mma_commit(smem_u32(&empty[s]));
        ++g;
      }
      if (!ok) break;
      mma_commit(smem_u32(&tfull[buf]));
      ++acc;
    }
    // every MMA issued by this thread has retired once `done` completes
    mma_commit(smem_u32(done));
    mbar_wait_bounded(smem_u32(done), 0, args.status, DRAIN_WAIT_NS);
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> FP64 global
    const int q = warp % 4;  // TMEM lane quarter accessible by this warp
    uint32_t acc = 0;
    for (int j = 0;; ++j) {
      const int slot = j % PS_RING;
      bool ok = mbar_wait_bounded(smem_u32(&sfull[slot]), (j / PS_RING) & 1, args.status, args.wait_ns);
      ok = __all_sync(0xffffffffu, ok);
      const int t = ok ? stile[slot] : -1, nk = ok ? snk[slot] : 0;
      __syncwarp();
      if (ok && lane == 0) mbar_arrive(smem_u32(&sempty[slot]));
      if (t < 0) break;
      const int z = t / mn;
      const int r = t - z * mn;
      const int ni = r / args.mt, mi = r - ni * args.mt;
      const int64_t m = (int64_t)mi * TC_BM + 32 * q + lane;
      const int64_t n0 = (int64_t)ni * BN;
      // element offset of C[m, n] (complex: interleaved real / imaginary parts)
      const int64_t cz = (int64_t)z * args.sC * (args.cplx ? 2 : 1);
      auto off = [&](int64_t n) -> int64_t {
        if (args.cplx) {
          const int64_t nn = n < args.Nlog ? n : n - args.Nlog;
          return cz + 2 * (m + args.ldc * nn) + (n < args.Nlog ? 0 : 1);
        }
        return cz + m + args.ldc * n;
      };
      const bool alpha_one = args.alpha == 1.0;
      auto store = [&](int64_t e, double val) {
        if (args.c_f32) {
          float* p = (float*)args.C + e;
          if (args.beta != 0.0) val = fma(args.beta, (double)*p, val);
          *p = (float)val;
        } else {
          double* p = args.C + e;
          if (args.beta != 0.0) val = fma(args.beta, *p, val);
          *p = val;
        }
      };
      if (nk == 0) {
        // no contributing k-block: C = beta * C
        if (m < args.M)
          for (int64_t n = n0; n < n0 + BN && n < args.N; ++n) store(off(n), 0.0);
        continue;
      }
      const uint32_t buf = acc & 1;
      ok = mbar_wait_bounded(smem_u32(&tfull[buf]), (acc >> 1) & 1, args.status, args.wait_ns);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      tc_fence_after();
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * BN + (uint32_t)c0;
        TMEM_LD32(taddr, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (m >= args.M) continue;
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const int64_t n = n0 + c0 + jj;
          if (n >= args.N) break;
          const double x = (double)__uint_as_float(v[jj]);
          store(off(n), alpha_one ? x : args.alpha * x);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&tempty[buf]));
      ++acc;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * BN));
  }
}

template <int BN, int STAGES>
constexpr int persistent_smem() {
  return STAGES * (TC_BM * 128 + BN * 128) + 1024 + 512;
}

// ------------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

static void load_encode() {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  if (!g_encode) throw Error(GB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
}

static CUtensorMap make_map(const Packed& P, int box_rows) {
  CUtensorMap m;
  const cuuint64_t es = (cuuint64_t)P.esz;
  cuuint64_t dims[3] = {(cuuint64_t)P.Kp, (cuuint64_t)P.rows, (cuuint64_t)(2 * P.batch)};
  cuuint64_t strides[2] = {(cuuint64_t)P.Kp * es, (cuuint64_t)P.Kp * P.rows * es};
  cuuint32_t box[3] = {(cuuint32_t)P.bk, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(&m, P.esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                       : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                        3, P.data, dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(GB_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return m;
}

// map over split planes [planes][rows][kdim] (K-major, 128-byte swizzle), box of one
// 128-byte K row by box_rows rows; used by the grouped sector-block GEMM
CUtensorMap make_plane_map(void* data, int esz, int64_t kdim, int64_t rows, int64_t planes,
                           int box_rows) {
  load_encode();
  GB_REQUIRE((kdim * esz) % 128 == 0 && ((uintptr_t)data % 256) == 0,
             "plane map: K rows must be whole 128-byte lines on an aligned buffer");
  CUtensorMap m;
  const cuuint64_t es = (cuuint64_t)esz;
  cuuint64_t dims[3] = {(cuuint64_t)kdim, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)kdim * es, (cuuint64_t)kdim * rows * es};
  cuuint32_t box[3] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(&m, esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                     : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                        3, data, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(GB_ERR_CUDA, "cuTensorMapEncodeTiled failed (plane map)");
  return m;
}

bool tc_available(gb_ctx* ctx) {
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx->device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx->device);
  return major == 10 && minor == 3;
}

void gemm_split(gb_ctx* ctx, int dtype, const Packed& A, const Packed& B, int64_t M,
                int64_t N, double alpha, double beta, void* C, int64_t ldc, int64_t sC,
                uint32_t* outmap, bool c_f32) {
  GB_REQUIRE(tc_available(ctx), "split-precision GEMM needs an sm_103 device");
  GB_REQUIRE(A.Kp == B.Kp && A.cplx == B.cplx && A.esz == B.esz,
             "gemm_split: operand packing mismatch");
  GB_REQUIRE(A.Kp % A.bk == 0, "gemm_split: Kp alignment");
  const bool tf32 = A.esz == 4;
  load_encode();
  static std::once_flag attr_once;  // contexts may launch from several host threads
  std::call_once(attr_once, [] {
    GB_CHECK_CUDA(cudaFuncSetAttribute(gemm_bf16x3_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       TC_SMEM_BYTES));
  });
  CUtensorMap ma = make_map(A, TC_BM);
  CUtensorMap mb = make_map(B, TC_BN);
  int64_t batch = std::max(A.batch, B.batch);
  GB_REQUIRE(A.batch == 1 || A.batch == batch, "gemm_split: batch mismatch (A)");
  GB_REQUIRE(B.batch == 1 || B.batch == batch, "gemm_split: batch mismatch (B)");
  int64_t Npk = B.rows;  // packed N (2N when complex)
  TcArgs a;
  a.M = M;
  a.N = Npk;
  a.Nlog = N;
  a.cplx = A.cplx;
  a.kblocks = (int)(A.Kp / TC_BK);
  a.batchA = (int)A.batch;
  a.batchB = (int)B.batch;
  a.alpha = alpha;
  a.beta = beta;
  a.C = (double*)C;
  a.ldc = ldc;
  a.sC = sC;
  a.status = ctx->d_status;
  a.wait_ns = ctx->wait_ns;
  GB_REQUIRE(M <= (int64_t)INT32_MAX && Npk <= (int64_t)INT32_MAX, "gemm_split: size");
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (ctx->profiling) {
    if (ctx->prof_used + 2 > ctx->prof_events.size()) {
      for (int i = 0; i < 64; ++i) {
        cudaEvent_t e;
        GB_CHECK_CUDA(cudaEventCreate(&e));
        ctx->prof_events.push_back(e);
      }
    }
    ev0 = ctx->prof_events[ctx->prof_used++];
    ev1 = ctx->prof_events[ctx->prof_used++];
    const double fl = (A.cplx ? 8.0 : 2.0) * (double)M * (double)N * (double)A.K;
    ctx->prof_flops += fl;
    ctx->prof_kind.push_back(0);
    ctx->prof_kind_flops[0] += fl;
    GB_CHECK_CUDA(cudaEventRecord(ev0, ctx->stream));
  }
  if (outmap) GB_REQUIRE(std::max(A.batch, B.batch) == 1, "gemm_split: output map needs batch 1");
  if (ctx->gemm_schedule == GB_SCHED_TILE && !tf32 && !outmap && !c_f32) {
    dim3 grid((unsigned)((M + TC_BM - 1) / TC_BM), (unsigned)((Npk + TC_BN - 1) / TC_BN),
              (unsigned)batch);
    GB_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "gemm_split: grid too large");
    gemm_bf16x3_kernel<<<grid, TC_THREADS, TC_SMEM_BYTES, ctx->stream>>>(ma, mb, a);
  } else {
    const int bn = ctx->gemm_bn ? ctx->gemm_bn : (Npk <= 128 ? 128 : 256);
    if (bn == 128) mb = make_map(B, 128);
    PArgs p;
    p.M = M;
    p.N = Npk;
    p.Nlog = N;
    p.cplx = A.cplx;
    p.kblocks = (int)(A.Kp / A.bk);
    p.mt = (int)((M + TC_BM - 1) / TC_BM);
    p.nt = (int)((Npk + bn - 1) / bn);
    const int64_t ntiles = (int64_t)p.mt * p.nt * batch;
    GB_REQUIRE(ntiles < (int64_t)INT32_MAX / 2, "gemm_split: too many tiles");
    p.ntiles = (int)ntiles;
    p.batchA = (int)A.batch;
    p.batchB = (int)B.batch;
    p.alpha = alpha;
    p.beta = beta;
    p.C = (double*)C;
    p.ldc = ldc;
    p.sC = sC;
    const bool masked = ctx->gemm_schedule != GB_SCHED_PERSISTENT_DENSE && A.mask && B.mask;
    GB_REQUIRE(!masked || A.kw == B.kw, "gemm_split: nonzero maps differ in width");
    p.maskA = masked ? A.mask : nullptr;
    p.maskB = masked ? B.mask : nullptr;
    p.kw = A.kw;
    p.mskA_b = A.mrows * A.kw;
    p.mskB_b = B.mrows * B.kw;
    p.mrowsB = B.mrows;
    p.counter = ctx->d_tile_counter;
    p.status = ctx->d_status;
    p.wait_ns = ctx->wait_ns;
    p.work = (ctx->profiling || ctx->counting) ? ctx->d_work : nullptr;
    p.outmap = outmap;
    p.prevmap = nullptr;
    p.onc = (N + 127) / 128;
    p.skip_zero_out = (outmap && !A.cplx) ? 1 : 0;
    p.c_f32 = c_f32 ? 1 : 0;
    if (outmap) {
      const size_t mb = outmap_bytes(M, N);
      if (p.skip_zero_out) {
        uint32_t* prev = outmap + mb / 4;
        GB_CHECK_CUDA(
            cudaMemcpyAsync(prev, outmap, mb, cudaMemcpyDeviceToDevice, ctx->stream));
        p.prevmap = prev;
      }
      GB_CHECK_CUDA(cudaMemsetAsync(outmap, 0, mb, ctx->stream));
    }
    GB_CHECK_CUDA(cudaMemsetAsync(ctx->d_tile_counter, 0, sizeof(unsigned int), ctx->stream));
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, std::max(1, ctx->num_sms));
#define GB_PERSISTENT(BN_, ST_, TF_)                                                          \
  do {                                                                                        \
    constexpr int SM = persistent_smem<BN_, ST_>();                                           \
    static std::once_flag once;                                                               \
    std::call_once(once, [] {                                                                 \
      GB_CHECK_CUDA(cudaFuncSetAttribute(gemm_bf16x3_persistent<BN_, ST_, TF_>,               \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SM));   \
    });                                                                                       \
    gemm_bf16x3_persistent<BN_, ST_, TF_><<<grid, TC_THREADS, SM, ctx->stream>>>(ma, mb, p); \
  } while (0)
    if (bn == 128) {
      if (tf32) GB_PERSISTENT(128, 6, true);
      else GB_PERSISTENT(128, 6, false);
    } else {
      if (tf32) GB_PERSISTENT(256, 4, true);
      else GB_PERSISTENT(256, 4, false);
    }
#undef GB_PERSISTENT
  }
  GB_CHECK_CUDA(cudaGetLastError());
  if (ev1) GB_CHECK_CUDA(cudaEventRecord(ev1, ctx->stream));
  count_launch(ctx);
  if (ctx->counting && A.cnt_valid && B.cnt_valid) {
    nonzero_products_kernel<<<256, 256, 0, ctx->stream>>>(A.cnt, B.cnt, A.Kp, batch,
                                                          A.batch > 1, B.batch > 1, ctx->d_work);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
  }
}

size_t outmap_bytes(int64_t M, int64_t N) {
  const int64_t bits = ((M + 127) / 128) * ((N + 127) / 128);
  return (size_t)((bits + 31) / 32) * 4;
}

// ------------------------------------------------------------------ unified entry
void gemm(gb_ctx* ctx, int prec, int dtype, char opA, char opB, int64_t M, int64_t N,
          int64_t K, double alpha, const void* A, int64_t lda, int64_t sA, const void* B,
          int64_t ldb, int64_t sB, double beta, void* C, int64_t ldc, int64_t sC,
          int64_t batch, const Packed* pA, const Packed* pB, uint32_t* outmap, bool c_f32) {
  if (M == 0 || N == 0 || batch == 0) return;
  GB_REQUIRE(!c_f32 || (prec != GB_PREC_FP64 && K > 0), "gemm: FP32 output only in split mode");
  if (prec == GB_PREC_FP64 || K == 0) {
    gemm_fp64(ctx, dtype, opA, opB, M, N, K, cplx{alpha, 0}, A, lda, sA, B, ldb, sB,
              cplx{beta, 0}, C, ldc, sC, batch);
    // every region written: a full output map
    if (outmap) GB_CHECK_CUDA(cudaMemsetAsync(outmap, 0xff, outmap_bytes(M, N), ctx->stream));
    return;
  }
  Packed a, b;
  if (pA) {
    a = *pA;
  } else {
    int64_t bA = (sA == 0) ? 1 : batch;
    void* dst =
        scratch(ctx, SLOT_PACK_A, packed_bytes(M, K, is_cplx(dtype), PACK_AS_A, bA, prec));
    pack_operand(ctx, dtype, PACK_AS_A, opA, M, K, A, lda, sA, bA, a, dst, prec);
  }
  if (pB) {
    b = *pB;
  } else {
    int64_t bB = (sB == 0) ? 1 : batch;
    void* dst =
        scratch(ctx, SLOT_PACK_B, packed_bytes(N, K, is_cplx(dtype), PACK_AS_B, bB, prec));
    pack_operand(ctx, dtype, PACK_AS_B, opB, N, K, B, ldb, sB, bB, b, dst, prec);
  }
  gemm_split(ctx, dtype, a, b, M, N, alpha, beta, C, ldc, sC, outmap, c_f32);
}

}  // namespace gb
