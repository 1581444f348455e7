// Split-precision GEMM on the 5th-generation tensor cores (sm_103a).
//
// Scheme ("bf16x3", a published split-operand scheme; see e.g. Henry, Tang & Heinecke,
// "Leveraging the bfloat16 Artificial Intelligence Datatype For Higher-Precision
// Computations", ARITH 2019): every FP64 operand x is split into hi = bf16(x) and
// lo = bf16(x - hi); the product is hi*hi + hi*lo + lo*hi accumulated in FP32.  The
// three products are one K-loop over (pair, k-block) that re-reads the hi/lo planes.
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
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound on any wait

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
__global__ void pack_kernel(PackArgs p, const double* __restrict__ src,
                            __nv_bfloat16* __restrict__ dst) {
  __shared__ double tre[32][33];
  __shared__ double tim[32][33];
  const int64_t b = blockIdx.z;
  src += b * p.stride * (p.cplx ? 2 : 1);
  __nv_bfloat16* hi = dst + b * 2 * p.rows * p.Kp;
  __nv_bfloat16* lo = hi + p.rows * p.Kp;
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
  for (int j = ty; j < 32; j += 8) {
    int64_t r = r0 + j, k = k0 + tx;
    if (r >= p.R || k >= p.Kh) continue;  // pads were zeroed by memset
    double re = tre[j][tx], im = tim[j][tx];
    auto put = [&](int64_t row, int64_t col, double v) {
      __nv_bfloat16 h = __double2bfloat16(v);
      __nv_bfloat16 l = __double2bfloat16(v - (double)__bfloat162float(h));
      hi[row * p.Kp + col] = h;
      lo[row * p.Kp + col] = l;
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
}

size_t packed_bytes(int64_t rows, int64_t K, bool cplx, int role, int64_t batch) {
  int64_t Kh = round_up(std::max<int64_t>(K, 1), KALIGN);
  int64_t Kp = cplx ? 2 * Kh : Kh;
  int64_t prow = (cplx && role == PACK_AS_B) ? 2 * rows : rows;
  return (size_t)batch * 2 * prow * Kp * 2;
}

void pack_operand(gb_ctx* ctx, int dtype, int role, char op, int64_t R, int64_t K,
                  const void* src, int64_t ld, int64_t stride, int64_t batch, Packed& out,
                  void* dst) {
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
  out.data = dst;
  out.rows = p.rows;
  out.Kp = p.Kp;
  out.K = K;
  out.Kh = p.Kh;
  out.batch = batch;
  out.cplx = cx;
  out.bytes = packed_bytes(R, K, cx, role, batch);
  // no memset: the kernel writes every (row, k < Kh) entry, zeros included for k >= K
  GB_REQUIRE(batch <= 65535 && (R + 31) / 32 <= 65535, "pack: grid too large");
  dim3 grid((unsigned)((p.Kh + 31) / 32), (unsigned)((R + 31) / 32), (unsigned)batch);
  pack_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>(p, (const double*)src,
                                                      (__nv_bfloat16*)dst);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

// ------------------------------------------------------------------ fused leg mix + pack
// y[a + out_off[J] + n*yn] = sum_e val[e] x[a + in_off[col[e]] + n*xn] written directly as
// the packed B operand of the following GEMM: logical B element (k, m) with
// k = a + kJ[J] (contraction index) and m = mJ[J] + n*mn (output column index).
template <bool CPLX>
__global__ void mixpack_kernel(int64_t A, int64_t N, int64_t xn, const int64_t* __restrict__ in_off,
                               const int64_t* __restrict__ kJ, const int64_t* __restrict__ mJ,
                               int64_t mn, const int* __restrict__ row_ptr,
                               const int* __restrict__ col, const double* __restrict__ val,
                               const double* __restrict__ x, __nv_bfloat16* __restrict__ hi,
                               int64_t Nlog, int64_t Kp, int64_t Kh, int64_t plane) {
  const int J = blockIdx.y;
  const int e0 = row_ptr[J], e1 = row_ptr[J + 1];
  __nv_bfloat16* lo = hi + plane;
  auto put = [&](int64_t row, int64_t c, double v) {
    __nv_bfloat16 h = __double2bfloat16(v);
    hi[row * Kp + c] = h;
    lo[row * Kp + c] = __double2bfloat16(v - (double)__bfloat162float(h));
  };
  for (int64_t n = blockIdx.z; n < N; n += gridDim.z) {
    const int64_t m = mJ[J] + n * mn;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < A;
         a += (int64_t)gridDim.x * blockDim.x) {
      const int64_t k = a + kJ[J];
      if (CPLX) {
        double re = 0.0, im = 0.0;
        for (int e = e0; e < e1; ++e) {
          const double* xv = x + 2 * (a + in_off[col[e]] + n * xn);
          double vr = val[2 * e], vi = val[2 * e + 1];
          re = fma(vr, xv[0], fma(-vi, xv[1], re));
          im = fma(vr, xv[1], fma(vi, xv[0], im));
        }
        put(m, k, re);
        put(m, Kh + k, -im);
        put(Nlog + m, k, im);
        put(Nlog + m, Kh + k, re);
      } else {
        double acc = 0.0;
        for (int e = e0; e < e1; ++e) acc = fma(val[e], x[a + in_off[col[e]] + n * xn], acc);
        put(m, k, acc);
      }
    }
  }
}

void mixpack_run(gb_ctx* ctx, const MixDev& m, const int64_t* kJ, const int64_t* mJ, int64_t mn,
                 int dtype, const void* x, Packed& out, int64_t Klog, int64_t Nlog) {
  const bool cx = is_cplx(dtype);
  GB_REQUIRE(m.nJ <= 65535, "mixpack: too many output rows");
  GB_REQUIRE(m.xa == 1, "mixpack: unit input stride required");
  // zero the K padding of every row once (entries k >= Klog are never produced by the mix)
  if (out.Kh > Klog) {
    __nv_bfloat16* base = (__nv_bfloat16*)out.data;
    const int64_t planes = 2 * out.batch;
    for (int64_t p = 0; p < planes; ++p) {
      char* pb = (char*)(base + p * out.rows * out.Kp);
      GB_CHECK_CUDA(cudaMemset2DAsync(pb + Klog * 2, out.Kp * 2, 0, (out.Kh - Klog) * 2, out.rows,
                                      ctx->stream));
      if (cx)
        GB_CHECK_CUDA(cudaMemset2DAsync(pb + (out.Kh + Klog) * 2, out.Kp * 2, 0,
                                        (out.Kh - Klog) * 2, out.rows, ctx->stream));
    }
  }
  dim3 grid((unsigned)std::min<int64_t>((m.A + 127) / 128, 64), (unsigned)m.nJ,
            (unsigned)std::min<int64_t>(m.N, 65535));
  const int64_t plane = out.rows * out.Kp;
  if (cx)
    mixpack_kernel<true><<<grid, 128, 0, ctx->stream>>>(
        m.A, m.N, m.xn, m.in_off, kJ, mJ, mn, m.row_ptr, m.col, m.val, (const double*)x,
        (__nv_bfloat16*)out.data, Nlog, out.Kp, out.Kh, plane);
  else
    mixpack_kernel<false><<<grid, 128, 0, ctx->stream>>>(
        m.A, m.N, m.xn, m.in_off, kJ, mJ, mn, m.row_ptr, m.col, m.val, (const double*)x,
        (__nv_bfloat16*)out.data, Nlog, out.Kp, out.Kh, plane);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: returns false (and records a timeout) when the bound expires
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int* status) {
  if (mbar_try_wait(bar, parity)) return true;
  unsigned long long t0 = globaltimer();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer() - t0 > WAIT_NS) {
      atomicExch(status, GB_ERR_TIMEOUT);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"((unsigned long long)map), "r"(bar), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                        // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                        // 128-byte swizzle
  return d;
}
// kind::f16 instruction descriptor: BF16 x BF16 -> F32, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

#define TMEM_LD32(taddr, r)                                                                   \
  asm volatile(                                                                               \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"      \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),  \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),           \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),        \
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),        \
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),        \
        "=r"(r[31])                                                                           \
      : "r"(taddr))

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
      ok = mbar_wait_bounded(smem_u32(&empty[s]), (round & 1) ^ 1, args.status);
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
        mbar_wait_bounded(smem_u32(&full[s]), (it / TC_STAGES) & 1, args.status);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    const uint32_t idesc = idesc_bf16(TC_BM, TC_BN);
    bool ok = true;
    for (int it = 0; it < total; ++it) {
      int s = it % TC_STAGES;
      ok = mbar_wait_bounded(smem_u32(&full[s]), (it / TC_STAGES) & 1, args.status);
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
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> FP64 global
    const int g = warp % 4;  // TMEM lane quarter accessible by this warp
    bool ok = mbar_wait_bounded(smem_u32(accum), 0, args.status);
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
        double v = args.alpha * (double)__uint_as_float(r[j]);
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
  cuuint64_t dims[3] = {(cuuint64_t)P.Kp, (cuuint64_t)P.rows, (cuuint64_t)(2 * P.batch)};
  cuuint64_t strides[2] = {(cuuint64_t)P.Kp * 2, (cuuint64_t)P.Kp * P.rows * 2};
  cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, P.data, dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(GB_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return m;
}

bool tc_available(gb_ctx* ctx) {
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx->device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx->device);
  return major == 10 && minor == 3;
}

void gemm_split(gb_ctx* ctx, int dtype, const Packed& A, const Packed& B, int64_t M,
                int64_t N, double alpha, double beta, void* C, int64_t ldc, int64_t sC) {
  GB_REQUIRE(tc_available(ctx), "split-precision GEMM needs an sm_103 device");
  GB_REQUIRE(A.Kp == B.Kp && A.cplx == B.cplx, "gemm_split: operand packing mismatch");
  GB_REQUIRE(A.Kp % TC_BK == 0, "gemm_split: Kp alignment");
  load_encode();
  static bool attr_set = false;
  if (!attr_set) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(gemm_bf16x3_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       TC_SMEM_BYTES));
    attr_set = true;
  }
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
  GB_REQUIRE(M <= (int64_t)INT32_MAX && Npk <= (int64_t)INT32_MAX, "gemm_split: size");
  dim3 grid((unsigned)((M + TC_BM - 1) / TC_BM), (unsigned)((Npk + TC_BN - 1) / TC_BN),
            (unsigned)batch);
  GB_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "gemm_split: grid too large");
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
    ctx->prof_flops += (A.cplx ? 8.0 : 2.0) * (double)M * (double)N * (double)A.K;
    GB_CHECK_CUDA(cudaEventRecord(ev0, ctx->stream));
  }
  gemm_bf16x3_kernel<<<grid, TC_THREADS, TC_SMEM_BYTES, ctx->stream>>>(ma, mb, a);
  GB_CHECK_CUDA(cudaGetLastError());
  if (ev1) GB_CHECK_CUDA(cudaEventRecord(ev1, ctx->stream));
  count_launch(ctx);
}

// ------------------------------------------------------------------ unified entry
void gemm(gb_ctx* ctx, int prec, int dtype, char opA, char opB, int64_t M, int64_t N,
          int64_t K, double alpha, const void* A, int64_t lda, int64_t sA, const void* B,
          int64_t ldb, int64_t sB, double beta, void* C, int64_t ldc, int64_t sC,
          int64_t batch, const Packed* pA, const Packed* pB) {
  if (M == 0 || N == 0 || batch == 0) return;
  if (prec == GB_PREC_FP64 || K == 0) {
    gemm_fp64(ctx, dtype, opA, opB, M, N, K, cplx{alpha, 0}, A, lda, sA, B, ldb, sB,
              cplx{beta, 0}, C, ldc, sC, batch);
    return;
  }
  Packed a, b;
  if (pA) {
    a = *pA;
  } else {
    int64_t bA = (sA == 0) ? 1 : batch;
    void* dst = scratch(ctx, SLOT_PACK_A, packed_bytes(M, K, is_cplx(dtype), PACK_AS_A, bA));
    pack_operand(ctx, dtype, PACK_AS_A, opA, M, K, A, lda, sA, bA, a, dst);
  }
  if (pB) {
    b = *pB;
  } else {
    int64_t bB = (sB == 0) ? 1 : batch;
    void* dst = scratch(ctx, SLOT_PACK_B, packed_bytes(N, K, is_cplx(dtype), PACK_AS_B, bB));
    pack_operand(ctx, dtype, PACK_AS_B, opB, N, K, B, ldb, sB, bB, b, dst);
  }
  gemm_split(ctx, dtype, a, b, M, N, alpha, beta, C, ldc, sC);
}

}  // namespace gb
