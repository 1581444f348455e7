// Grouped split-precision GEMM over U(1) sector blocks (sm_103a).
//
// TensorKit runs every contraction of a symmetric TensorMap block by block: one dense
// GEMM per coupled charge (the per-sector `mul!` behind each `@plansor` of
// src/algorithms/derivatives/hamiltonian_derivatives.jl:485-500).  Here the same block
// structure is read off the charge labels of the GEMM's three index spaces (grouped.h),
// and all blocks of one contraction run in ONE persistent launch:
//
//  * operands are packed block-stacked (gpack_kernel): group g owns the rows of its M (or
//    N) members, its K members sit in columns [0, kpad_g) of a K-major hi/lo plane pair,
//    padded with zeros to a multiple of 64; nothing outside the blocks is stored;
//  * a host-built tile list covers each block with 128-row tiles along the kernel's M and
//    a per-group MMA width (multiple of 16, <= 256) along N, so a block of 272 columns
//    runs two tiles of 144, not two of 256; tiles are handed out longest first;
//  * the kernel is the persistent warp-specialised tcgen05 GEMM of gemm_tc.cu (TMA
//    producer, single-thread MMA issuer, TMEM double-buffered accumulator, four epilogue
//    warps) with per-tile K length and N width; rows and columns that belong to the next
//    group are computed but never stored;
//  * the epilogue writes element (m, n) of a tile to C[rowoff[m] + coloff[n]] -- its place
//    in the charge-sorted dense embedding -- directly when consecutive rows are adjacent in
//    memory, or after a transpose through shared memory when consecutive columns are.
//
// The orientation of every GEMM is chosen per plan: the kernel's M (granularity 128) takes
// whichever side wastes less, the other side gets the fine N granularity.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <numeric>
#include <type_traits>

#include "grouped.h"
#include "tc_ptx.cuh"

namespace gb {

CUtensorMap make_plane_map(void* data, int esz, int64_t kdim, int64_t rows, int64_t planes,
                           int box_rows);
bool tc_available(gb_ctx* ctx);

namespace {
constexpr int G_BM = 128;
constexpr int G_BN = 256;     // widest tile (TMEM: two accumulators of 256 columns)
constexpr int G_BOXN = 64;    // rows per TMA box of the B operand
constexpr int G_KPAD = 64;    // K padding of every group (one BF16 K-block, two TF32)
constexpr int G_RING = 4;
constexpr int G_THREADS = 192;
inline int64_t rup(int64_t x, int64_t m) { return (x + m - 1) / m * m; }
}  // namespace

// ------------------------------------------------------------------ labels and plans
std::vector<int32_t> leg_labels(const std::vector<LegSpec>& legs,
                                const std::vector<const int32_t*>& q) {
  int64_t n = 1;
  for (const LegSpec& l : legs) n *= l.n;
  std::vector<int32_t> lab((size_t)n, 0);
  int64_t stride = 1;
  for (const LegSpec& l : legs) {
    const int32_t* c = (l.which > Q_NONE && l.which < Q_COUNT) ? q[l.which] : nullptr;
    if (c) {
      // index i = inner + stride * (j + l.n * outer): leg value j, no divisions
      for (int64_t base = 0; base < n; base += stride * l.n)
        for (int64_t j = 0; j < l.n; ++j) {
          const int32_t ch = c[j];
          int32_t* dst = lab.data() + base + stride * j;
          for (int64_t i = 0; i < stride; ++i) {
            if (dst[i] == NO_LABEL) continue;
            dst[i] = (ch == NO_LABEL) ? NO_LABEL : dst[i] + l.sign * ch;
          }
        }
    }
    stride *= l.n;
  }
  return lab;
}

void gplan_build(GPlan& p, const std::vector<int32_t>& labM, const std::vector<int32_t>& labK,
                 const std::vector<int32_t>& labN, bool first_writer, int64_t ldc, int sms) {
  p = GPlan();
  // labels are small integers (sums of charges): count them in dense arrays over their range
  int32_t lo = INT32_MAX, hi = INT32_MIN;
  for (const auto* lab : {&labM, &labN, &labK})
    for (int32_t v : *lab)
      if (v != NO_LABEL) {
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
  const int64_t span = hi >= lo ? (int64_t)hi - lo + 1 : 0;
  std::vector<int64_t> cntM(span, 0), cntN(span, 0), cntK(span, 0);
  for (int32_t v : labM)
    if (v != NO_LABEL) ++cntM[v - lo];
  for (int32_t v : labN)
    if (v != NO_LABEL) ++cntN[v - lo];
  for (int32_t v : labK)
    if (v != NO_LABEL) ++cntK[v - lo];
  std::vector<int32_t> gid(span, -1);  // label - lo -> group
  for (int64_t t = 0; t < span; ++t) {
    if (!cntM[t] || !cntN[t]) continue;
    if (!cntK[t] && !first_writer) continue;
    gid[t] = (int32_t)p.label.size();
    p.label.push_back((int32_t)(t + lo));
  }
  p.G = (int)p.label.size();
  const int G = p.G;
  // members of every group in increasing dense order
  auto members = [&](const std::vector<int32_t>& lab, std::vector<int32_t>& dense,
                     std::vector<int32_t>& start) {
    std::vector<int32_t> g_of(lab.size(), -1);
    start.assign(G + 1, 0);
    for (size_t i = 0; i < lab.size(); ++i) {
      if (lab[i] == NO_LABEL) continue;
      const int32_t g = gid[lab[i] - lo];
      if (g < 0) continue;
      g_of[i] = g;
      ++start[g + 1];
    }
    for (int g = 0; g < G; ++g) start[g + 1] += start[g];
    dense.assign(start[G], 0);
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (size_t i = 0; i < lab.size(); ++i)
      if (g_of[i] >= 0) dense[fill[g_of[i]]++] = (int32_t)i;
  };
  members(labM, p.side[0].dense, p.side[0].gstart);
  members(labN, p.side[1].dense, p.side[1].gstart);
  members(labK, p.kdense, p.kstart);
  p.kpad.assign(G, 0);
  p.kmax = G_KPAD;
  for (int g = 0; g < G; ++g) {
    p.kpad[g] = (int32_t)rup(p.kstart[g + 1] - p.kstart[g], G_KPAD);
    p.kmax = std::max<int64_t>(p.kmax, p.kpad[g]);
  }
  auto cnt = [&](int s, int g) -> int64_t { return p.side[s].gstart[g + 1] - p.side[s].gstart[g]; };
  // orientation: the kernel's rows come in tiles of 128, its columns in steps of 16
  double cost[2] = {0.0, 0.0};
  for (int g = 0; g < G; ++g) {
    const double kk = std::max<int64_t>(p.kpad[g], G_KPAD);
    cost[0] += (double)rup(cnt(0, g), G_BM) * (double)rup(cnt(1, g), 16) * kk;
    cost[1] += (double)rup(cnt(1, g), G_BM) * (double)rup(cnt(0, g), 16) * kk;
  }
  p.trans = cost[1] < 0.9 * cost[0];
  const int sa = p.trans ? 1 : 0, sb = 1 - sa;
  for (int g = 0; g < G; ++g) {
    const int64_t Mg = cnt(sa, g), Ng = cnt(sb, g), Kg = p.kstart[g + 1] - p.kstart[g];
    p.block_flops += 2.0 * (double)cnt(0, g) * (double)cnt(1, g) * (double)Kg;
    if (Mg == 0 || Ng == 0) continue;
    const int64_t ntn = (Ng + G_BN - 1) / G_BN;
    const int64_t w = rup((Ng + ntn - 1) / ntn, 16);
    for (int64_t mi = 0; mi < Mg; mi += G_BM)
      for (int64_t ni = 0; ni < Ng; ni += w) {
        GTile t;
        t.m0 = (int32_t)(p.side[sa].gstart[g] + mi);
        t.n0 = (int32_t)(p.side[sb].gstart[g] + ni);
        t.nkb = p.kpad[g] / G_KPAD;
        t.nw = (int32_t)std::min<int64_t>(w, rup(Ng - ni, 16));
        t.mlim = p.side[sa].gstart[g + 1];
        t.nlim = p.side[sb].gstart[g + 1];
        t.g = g;
        t.kb0 = 0;
        t.nsplit = 1;
        t.sid = 0;
        t.pslot = -1;
        t.cslot = -1;
        p.tiles.push_back(t);
        p.tile_flops += 2.0 * G_BM * (double)t.nw * (double)p.kpad[g];
      }
  }
  // split K: a tile longer than the target runs as several units, so that the long tiles
  // of a plan with few tiles still spread over every multiprocessor
  {
    int64_t total = 0;
    for (const GTile& t : p.tiles) total += t.nkb;
    const int64_t target = std::max<int64_t>(8, (total + 2 * sms - 1) / (2 * std::max(sms, 1)));
    std::vector<GTile> units;
    for (const GTile& t : p.tiles) {
      if (t.nkb <= target + target / 2) {
        units.push_back(t);
        continue;
      }
      const int ns = (int)((t.nkb + target - 1) / target);
      const int per = (t.nkb + ns - 1) / ns;
      int kb = 0, sid = 0;
      const int first = p.nslots;
      for (; kb < t.nkb; kb += per, ++sid) {
        GTile u = t;
        u.kb0 = kb;
        u.nkb = std::min(per, t.nkb - kb);
        u.sid = sid;
        u.pslot = first;
        u.cslot = p.ncounters;
        units.push_back(u);
      }
      for (size_t i = units.size() - sid; i < units.size(); ++i) units[i].nsplit = sid;
      p.nslots += sid;
      ++p.ncounters;
    }
    p.tiles.swap(units);
  }
  // longest tiles first: the persistent kernel hands them out in this order
  std::stable_sort(p.tiles.begin(), p.tiles.end(), [](const GTile& a, const GTile& b) {
    return (int64_t)a.nkb * a.nw > (int64_t)b.nkb * b.nw;
  });
  for (int s = 0; s < 2; ++s) {
    GSide& sd = p.side[s];
    sd.rows_alloc = rup(std::max<int64_t>((int64_t)sd.dense.size(), 1), G_BM);
    for (int g = 0; g < G; ++g)
      for (int32_t r = sd.gstart[g]; r < sd.gstart[g + 1]; r += 32)
        for (int32_t k = 0; k < p.kpad[g]; k += 32)
          sd.ptiles.push_back(GPackTile{r, std::min<int32_t>(32, sd.gstart[g + 1] - r), g, k});
  }
  // C is column-major: element (m, n) at m + ldc * n (offsets built in gplan_upload)
  p.ldc = ldc;
}

namespace {
struct Blob {
  std::vector<char> h;
  size_t add(const void* src, size_t bytes) {
    const size_t off = rup((int64_t)h.size(), 256);
    h.resize(off + std::max<size_t>(bytes, 16), 0);
    if (bytes) memcpy(h.data() + off, src, bytes);
    return off;
  }
};
}  // namespace

void gplan_upload(gb_ctx* ctx, GPlan& p, const std::function<void*(size_t)>& alloc) {
  const int sa = p.trans ? 1 : 0, sb = 1 - sa;
  auto offs = [&](int s) {
    const bool is_m = (s == 0);  // M members are output rows, N members output columns
    std::vector<int64_t> o(p.side[s].dense.size());
    for (size_t i = 0; i < o.size(); ++i)
      o[i] = is_m ? (int64_t)p.side[s].dense[i] : p.ldc * (int64_t)p.side[s].dense[i];
    return o;
  };
  const std::vector<int64_t> ro = offs(sa), co = offs(sb);
  std::vector<int32_t> klen(p.G);
  for (int g = 0; g < p.G; ++g) klen[g] = p.kstart[g + 1] - p.kstart[g];
  Blob b;
  const size_t o_t = b.add(p.tiles.data(), p.tiles.size() * sizeof(GTile));
  const size_t o_r = b.add(ro.data(), ro.size() * 8);
  const size_t o_c = b.add(co.data(), co.size() * 8);
  size_t o_d[2], o_g[2], o_p[2];
  for (int s = 0; s < 2; ++s) {
    o_d[s] = b.add(p.side[s].dense.data(), p.side[s].dense.size() * 4);
    o_g[s] = b.add(p.side[s].gstart.data(), p.side[s].gstart.size() * 4);
    o_p[s] = b.add(p.side[s].ptiles.data(), p.side[s].ptiles.size() * sizeof(GPackTile));
  }
  const size_t o_kd = b.add(p.kdense.data(), p.kdense.size() * 4);
  const size_t o_ks = b.add(p.kstart.data(), p.kstart.size() * 4);
  const size_t o_kl = b.add(klen.data(), klen.size() * 4);
  const size_t arrive_bytes = (size_t)std::max(p.ncounters, 1) * sizeof(unsigned int);
  const size_t o_cnt = (b.h.size() + 255) / 256 * 256;
  b.h.resize(o_cnt + arrive_bytes, 0);  // zeroed: every counter starts at 0
  char* d = (char*)alloc(b.h.size());
  p.dev = d;
  GB_CHECK_CUDA(cudaMemcpyAsync(d, b.h.data(), b.h.size(), cudaMemcpyHostToDevice, ctx->stream));
  // the host staging buffer dies with this scope: finish the copy first
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  p.d_tiles = (GTile*)(d + o_t);
  p.d_rowoff = (int64_t*)(d + o_r);
  p.d_coloff = (int64_t*)(d + o_c);
  for (int s = 0; s < 2; ++s) {
    p.d_dense[s] = (int32_t*)(d + o_d[s]);
    p.d_gstart[s] = (int32_t*)(d + o_g[s]);
    p.d_ptiles[s] = (GPackTile*)(d + o_p[s]);
  }
  p.d_kdense = (int32_t*)(d + o_kd);
  p.d_kstart = (int32_t*)(d + o_ks);
  p.d_klen = (int32_t*)(d + o_kl);
  p.d_arrive = (unsigned int*)(d + o_cnt);
  p.d_partial = nullptr;
  if (p.nslots > 0)
    p.d_partial = (float*)alloc((size_t)p.nslots * G_BM * G_BN * sizeof(float));
}

size_t goperand_bytes(const GPlan& p, int side, int prec) {
  const int esz = prec == GB_PREC_TF32X3 ? 4 : 2;
  return (size_t)2 * p.side[side].rows_alloc * p.kmax * esz;
}

void goperand_init(gb_ctx* ctx, GOperand& op, const GPlan& p, int side, void* data, int prec) {
  op.esz = prec == GB_PREC_TF32X3 ? 4 : 2;
  op.rows = p.side[side].rows_alloc;
  op.kmax = p.kmax;
  op.data = data;
  op.bytes = goperand_bytes(p, side, prec);
  // every entry a kernel may read is defined: blocks are (re)packed in full, the rest is
  // never written again
  GB_CHECK_CUDA(cudaMemsetAsync(data, 0, op.bytes, ctx->stream));
}

// ------------------------------------------------------------------ packing
template <typename E>
__global__ void gpack_kernel(const GPackTile* __restrict__ tiles, const int32_t* __restrict__ rdense,
                             const int32_t* __restrict__ kdense, const int32_t* __restrict__ kstart,
                             const int32_t* __restrict__ klen, const double* __restrict__ src,
                             int64_t rs, int64_t ks, int rowfast, E* __restrict__ hi,
                             int64_t plane, int64_t kmax, unsigned long long* nnz, int64_t klo,
                             int64_t khi) {
  __shared__ float t[32][33];
  __shared__ unsigned char in[32];  // column in this pack's K range
  const GPackTile T = tiles[blockIdx.x];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int32_t kl = klen[T.g], k0 = kstart[T.g];
  const bool full = klo == 0 && khi == INT64_MAX;
  if (ty == 0) {
    const int kp = T.kp0 + tx;
    bool inr = full;
    if (kp < kl) {
      const int64_t kd = kdense[k0 + kp];
      inr = kd >= klo && kd < khi;
    }
    in[tx] = inr ? 1 : 0;
  }
  __syncthreads();
  // load with the source's contiguous index on threadIdx.x; the planes keep at most 22 bits,
  // so the value is rounded to FP32 once and split there
  for (int j = ty; j < 32; j += 8) {
    const int i = rowfast ? tx : j;    // row within the block
    const int kk = rowfast ? j : tx;   // column within the block
    const int kp = T.kp0 + kk;
    float v = 0.0f;
    if (i < T.nr && kp < kl && in[kk])
      v = (float)src[(int64_t)rdense[T.rp0 + i] * rs + ((int64_t)kdense[k0 + kp] - klo) * ks];
    t[i][kk] = v;
  }
  __syncthreads();
  E* lo = hi + plane;
  int nz = 0;
  if (in[tx])
    for (int i = ty; i < T.nr; i += 8) {
      const float v = t[i][tx];
      nz += (v != 0.0f);
      split_put_f(hi, lo, (int64_t)(T.rp0 + i) * kmax + T.kp0 + tx, v);
    }
  if (nnz) {
    for (int o = 16; o > 0; o >>= 1) nz += __shfl_down_sync(0xffffffffu, nz, o);
    if ((threadIdx.x & 31) == 0 && nz) atomicAdd(nnz, (unsigned long long)nz);
  }
}

// nonzero entries (r, k) of a dense operand whose row and column labels differ (or are
// undefined): entries a block-diagonal contraction would silently drop
__global__ void label_violation_kernel(const double* __restrict__ src, int64_t R, int64_t K,
                                       int64_t rs, int64_t ks, const int32_t* __restrict__ labR,
                                       const int32_t* __restrict__ labK,
                                       unsigned long long* bad) {
  unsigned long long c = 0;
  // blocks over the slow index, threads over the fast one: consecutive threads read
  // consecutive addresses, no index division
  const bool rfast = rs == 1;
  const int64_t F = rfast ? R : K, S = rfast ? K : R;
  const int64_t fstr = rfast ? rs : ks, sstr = rfast ? ks : rs;
  const int32_t* labF = rfast ? labR : labK;
  const int32_t* labS = rfast ? labK : labR;
  for (int64_t sl = blockIdx.x; sl < S; sl += gridDim.x) {
    const int32_t b = labS[sl];
    const double* col = src + sl * sstr;
    for (int64_t f = threadIdx.x; f < F; f += blockDim.x) {
      if (col[f * fstr] == 0.0) continue;
      const int32_t a = labF[f];
      c += (a == NO_LABEL || b == NO_LABEL || a != b);
    }
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(bad, c);
}

__global__ void dense_nnz_kernel(const double* __restrict__ src, int64_t rows, int64_t cols,
                                 int64_t ld, unsigned long long* nnz) {
  unsigned long long c = 0;
  const int64_t n = rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    c += (src[(i % rows) + ld * (i / rows)] != 0.0);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(nnz, c);
}

static unsigned long long* nnz_counter(gb_ctx* ctx) {
  unsigned long long* d = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(&d, sizeof(unsigned long long), ctx->stream));
  GB_CHECK_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  return d;
}
static int64_t nnz_read(gb_ctx* ctx, unsigned long long* d) {
  unsigned long long h = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  GB_CHECK_CUDA(cudaFreeAsync(d, ctx->stream));
  return (int64_t)h;
}

int64_t gpack(gb_ctx* ctx, const GPlan& p, int side, const double* src, int64_t rs, int64_t ks,
              GOperand& op, bool count_nnz, int64_t klo, int64_t khi) {
  const GSide& sd = p.side[side];
  if (sd.ptiles.empty()) return 0;
  unsigned long long* cnt = count_nnz ? nnz_counter(ctx) : nullptr;
  const int rowfast = (rs == 1) ? 1 : 0;
  const int64_t plane = op.rows * op.kmax;
  const unsigned grid = (unsigned)sd.ptiles.size();
  if (op.esz == 4)
    gpack_kernel<float><<<grid, dim3(32, 8), 0, ctx->stream>>>(
        p.d_ptiles[side], p.d_dense[side], p.d_kdense, p.d_kstart, p.d_klen, src, rs, ks,
        rowfast, (float*)op.data, plane, op.kmax, cnt, klo, khi);
  else
    gpack_kernel<__nv_bfloat16><<<grid, dim3(32, 8), 0, ctx->stream>>>(
        p.d_ptiles[side], p.d_dense[side], p.d_kdense, p.d_kstart, p.d_klen, src, rs, ks,
        rowfast, (__nv_bfloat16*)op.data, plane, op.kmax, cnt, klo, khi);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  return cnt ? nnz_read(ctx, cnt) : 0;
}

int64_t label_violations(gb_ctx* ctx, const double* src, int64_t R, int64_t K, int64_t rs,
                         int64_t ks, const std::vector<int32_t>& labR,
                         const std::vector<int32_t>& labK) {
  if (R <= 0 || K <= 0) return 0;
  GB_REQUIRE((int64_t)labR.size() == R && (int64_t)labK.size() == K, "labels: size mismatch");
  int32_t* d = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(&d, (R + K) * sizeof(int32_t), ctx->stream));
  GB_CHECK_CUDA(cudaMemcpyAsync(d, labR.data(), R * sizeof(int32_t), cudaMemcpyHostToDevice,
                                ctx->stream));
  GB_CHECK_CUDA(cudaMemcpyAsync(d + R, labK.data(), K * sizeof(int32_t), cudaMemcpyHostToDevice,
                                ctx->stream));
  unsigned long long* cnt = nnz_counter(ctx);
  const int64_t slow = rs == 1 ? K : R;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(slow, 152 * 16));
  label_violation_kernel<<<grid, 256, 0, ctx->stream>>>(src, R, K, rs, ks, d, d + R, cnt);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  const int64_t bad = nnz_read(ctx, cnt);  // synchronises: the label copies are done
  GB_CHECK_CUDA(cudaFreeAsync(d, ctx->stream));
  return bad;
}

int64_t dense_nnz(gb_ctx* ctx, const double* src, int64_t rows, int64_t cols, int64_t ld) {
  if (rows <= 0 || cols <= 0) return 0;
  unsigned long long* cnt = nnz_counter(ctx);
  const unsigned grid = (unsigned)std::min<int64_t>((rows * cols + 255) / 256, 152 * 16);
  dense_nnz_kernel<<<grid, 256, 0, ctx->stream>>>(src, rows, cols, ld, cnt);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  return nnz_read(ctx, cnt);
}

// ------------------------------------------------------------------ the AA mix
// one warp per (output row J, column n): the lanes walk the row's l' range 32 at a time, so
// reads of the FP32 intermediate and writes of the packed planes are both contiguous
template <typename E>
__global__ void gmix_kernel(int64_t nJ, int64_t N, int64_t xn, const int64_t* __restrict__ in_off,
                            const int* __restrict__ row_ptr, const int* __restrict__ col,
                            const double* __restrict__ val, const float* __restrict__ x,
                            const GMixEntry* __restrict__ ent, E* __restrict__ hi, int64_t plane,
                            int64_t kmax) {
  const int J = blockIdx.y;
  const int e0 = row_ptr[J], e1 = row_ptr[J + 1];
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  E* lo = hi + plane;
  for (int64_t n = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); n < N;
       n += warps) {
    const GMixEntry en = ent[n * nJ + J];
    if (en.hi <= en.lo || en.row < 0) continue;
    const int64_t base = (int64_t)en.row * kmax + en.kst - en.lo;
    // eight 32-element chunks per pass with their loads issued together (more bytes in
    // flight per warp: the mix is a short strided copy when its rows hold one entry)
    constexpr int U = 8;
    for (int64_t a0 = en.lo + lane; a0 < en.hi; a0 += 32 * U) {
      // the arithmetic of gmix_staged_kernel, term for term (identical results)
      float s[U], c[U];
#pragma unroll
      for (int u = 0; u < U; ++u) s[u] = c[u] = 0.0f;
      for (int e = e0; e < e1; ++e) {
        const float* xp = x + in_off[col[e]] + n * xn;
        float xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t a = a0 + 32 * u;
          xv[u] = a < en.hi ? xp[a] : 0.0f;
        }
        const float vh = (float)val[e];
        const float vl = (float)(val[e] - (double)vh);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (std::is_same<E, float>::value) {
            const float p = vh * xv[u];
            const float pe = fmaf(vh, xv[u], -p) + vl * xv[u];
            const float t = s[u] + p, z = t - s[u];
            c[u] += ((s[u] - (t - z)) + (p - z)) + pe;
            s[u] = t;
          } else {
            s[u] = fmaf(vh, xv[u], s[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t a = a0 + 32 * u;
        if (a < en.hi) split_put_f(hi, lo, base + a, s[u] + c[u]);
      }
    }
  }
}

void gmix_run(gb_ctx* ctx, const MixDev& m, const GMixEntry* ent, int64_t span_max,
              const float* t1, GOperand& out) {
  GB_REQUIRE(!m.cplx && m.xa == 1, "grouped mix: real data with unit input stride");
  GB_REQUIRE(m.nJ <= 65535, "grouped mix: too many output rows");
  (void)span_max;
  // 8 warps per block, one (J, n) pair per warp
  dim3 grid((unsigned)std::min<int64_t>((m.N + 7) / 8, 1024), (unsigned)m.nJ);
  const int64_t plane = out.rows * out.kmax;
  if (out.esz == 4)
    gmix_kernel<float><<<grid, 256, 0, ctx->stream>>>(m.nJ, m.N, m.xn, m.in_off, m.row_ptr,
                                                      m.col, m.val, t1, ent, (float*)out.data,
                                                      plane, out.kmax);
  else
    gmix_kernel<__nv_bfloat16><<<grid, 256, 0, ctx->stream>>>(
        m.nJ, m.N, m.xn, m.in_off, m.row_ptr, m.col, m.val, t1, ent,
        (__nv_bfloat16*)out.data, plane, out.kmax);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

template <typename E>
__global__ void gmix_staged_kernel(int NL, int64_t nJ, int64_t xn, const int64_t* __restrict__ in_off,
                                   const int* __restrict__ grp, const int* __restrict__ gli,
                                   const float* __restrict__ gvh, const float* __restrict__ gvl,
                                   const int* __restrict__ rstart, const int* __restrict__ cstart,
                                   const float* __restrict__ x, const GMixEntry* __restrict__ ent,
                                   const int2* __restrict__ rng, const int* __restrict__ jlist,
                                   const int* __restrict__ jstart, const int* __restrict__ ilist,
                                   const int* __restrict__ istart, int chunk, int csr_floats,
                                   E* __restrict__ hi, int64_t plane, int64_t kmax) {
  constexpr bool TF = std::is_same<E, float>::value;
  constexpr int RA = 4;  // 32-lane columns per thread
  extern __shared__ float sm[];
  const int g = blockIdx.y;
  const int64_t n = blockIdx.x;
  const int2 r = rng[n * NL + g];
  if (r.y <= r.x) return;
  const int i0 = istart[g], ni = istart[g + 1] - i0;
  const int j0 = jstart[g], nj = jstart[g + 1] - j0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // the group's rows in shared memory: row pointers, local input index, coefficient hi (lo)
  const int e0 = cstart[g], ne = cstart[g + 1] - e0;
  int* rp = (int*)sm;
  int* li = rp + nj + 1;
  float* vh = (float*)(li + ne);
  float* vl = vh + ne;
  float* stage = sm + csr_floats;
  for (int k = threadIdx.x; k <= nj; k += blockDim.x) rp[k] = grp[rstart[g] + k] - e0;
  for (int k = threadIdx.x; k < ne; k += blockDim.x) {
    li[k] = gli[e0 + k];
    vh[k] = gvh[e0 + k];
    if (TF) vl[k] = gvl[e0 + k];
  }
  E* lo = hi + plane;
  // base offset of every staged input of this column (one dependent lookup per input)
  int64_t* ibase = (int64_t*)(stage + ni * chunk + (ni * chunk & 1));
  for (int i = threadIdx.x; i < ni; i += blockDim.x) ibase[i] = in_off[ilist[i0 + i]] + n * xn;
  __syncthreads();
  for (int a0 = r.x; a0 < r.y; a0 += chunk) {
    const int w = min(chunk, r.y - a0);
#pragma unroll 4
    for (int idx = threadIdx.x; idx < ni * w; idx += blockDim.x) {
      const int i = idx / w, a = idx - i * w;
      stage[idx] = x[(int64_t)(a0 + a) + ibase[i]];
    }
    __syncthreads();
    for (int jj = warp; jj < nj; jj += nw) {
      const GMixEntry en = ent[n * nJ + jlist[j0 + jj]];
      if (en.row < 0) continue;
      const int64_t base = (int64_t)en.row * kmax + en.kst - en.lo;
      const int b0 = rp[jj], b1 = rp[jj + 1];
      for (int ab = 0; ab < w; ab += 32 * RA) {
        float s[RA], c[RA];
#pragma unroll
        for (int k = 0; k < RA; ++k) s[k] = c[k] = 0.0f;
        for (int e = b0; e < b1; ++e) {
          const float* xr = stage + li[e] * w + ab + lane;
          const float h = vh[e];
#pragma unroll
          for (int k = 0; k < RA; ++k) {
            const float xv = (ab + lane + 32 * k < w) ? xr[32 * k] : 0.0f;
            if (TF) {
              const float p = h * xv;
              const float pe = fmaf(h, xv, -p) + vl[e] * xv;
              const float t = s[k] + p, z = t - s[k];
              c[k] += ((s[k] - (t - z)) + (p - z)) + pe;
              s[k] = t;
            } else {
              s[k] = fmaf(h, xv, s[k]);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < RA; ++k) {
          const int a = ab + lane + 32 * k;
          if (a < w) split_put_f(hi, lo, base + a0 + a, s[k] + c[k]);
        }
      }
    }
    __syncthreads();
  }
}

void gmix_staged_run(gb_ctx* ctx, const MixDev& m, const GMixStaged& g, const GMixEntry* ent,
                     const float* t1, GOperand& out) {
  GB_REQUIRE(!m.cplx && m.xa == 1, "grouped mix: real data with unit input stride");
  GB_REQUIRE(g.NL <= 65535 && m.N <= 0x7fffffff, "grouped mix: grid too large");
  dim3 grid((unsigned)m.N, (unsigned)g.NL);
  const int64_t plane = out.rows * out.kmax;
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(gmix_staged_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         96 * 1024);
    cudaFuncSetAttribute(gmix_staged_kernel<__nv_bfloat16>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
  });
  GB_REQUIRE(g.smem <= 96 * 1024 && g.smem_tf32 <= 96 * 1024,
             "grouped mix: staging buffer too large");
  if (out.esz == 4)
    gmix_staged_kernel<float><<<grid, 256, g.smem_tf32, ctx->stream>>>(
        g.NL, m.nJ, m.xn, m.in_off, g.rp, g.li, g.vh, g.vl, g.rstart, g.cstart, t1, ent, g.rng,
        g.jlist, g.jstart, g.ilist, g.istart, g.chunk_tf32, g.csr_floats_tf32, (float*)out.data,
        plane, out.kmax);
  else
    gmix_staged_kernel<__nv_bfloat16><<<grid, 256, g.smem, ctx->stream>>>(
        g.NL, m.nJ, m.xn, m.in_off, g.rp, g.li, g.vh, g.vl, g.rstart, g.cstart, t1, ent, g.rng,
        g.jlist, g.jstart, g.ilist, g.istart, g.chunk, g.csr_floats, (__nv_bfloat16*)out.data,
        plane, out.kmax);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

// ------------------------------------------------------------------ the grouped kernel
struct GArgs {
  const GTile* tiles;
  int ntiles;
  int trans_store;  // consecutive output columns (not rows) are adjacent in memory
  const int64_t* rowoff;
  const int64_t* coloff;
  double alpha, beta;
  void* C;
  int c_f32;
  unsigned int* counter;
  int* status;
  unsigned long long wait_ns;
  double* work;
  float* partial;         // split-K partial sums [slot][G_BN][128]
  unsigned int* arrive;   // split-K arrival counters
};

template <int STAGES>
constexpr int grouped_smem() {
  return STAGES * (G_BM * 128 + G_BN * 128) + 4 * 32 * 33 * 4 + 1024 + 512;
}

template <int STAGES, bool TF32>
__global__ void __launch_bounds__(G_THREADS, 1)
    gemm_grouped_kernel(const __grid_constant__ CUtensorMap mapA,
                        const __grid_constant__ CUtensorMap mapB, GArgs args) {
  constexpr int BKE = TF32 ? 32 : 64;        // K elements per stage (one 128-byte row)
  constexpr int KB_PER_PAD = G_KPAD / BKE;   // stages per padded K unit
  constexpr int A_BYTES = G_BM * 128;
  constexpr int B_BYTES = G_BN * 128;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr int BOX_BYTES = G_BOXN * 128;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* xbuf = (float*)(smem + STAGES * STAGE_BYTES);  // [4 warps][32][33] transposes
  uint64_t* bars = (uint64_t*)(xbuf + 4 * 32 * 33);
  uint64_t* full = bars;                 // [STAGES]  TMA -> MMA
  uint64_t* empty = full + STAGES;       // [STAGES]  MMA -> TMA
  uint64_t* tfull = empty + STAGES;      // [2]       MMA -> epilogue
  uint64_t* tempty = tfull + 2;          // [2]       epilogue -> MMA
  uint64_t* sfull = tempty + 2;          // [RING]    scheduler -> consumers
  uint64_t* sempty = sfull + G_RING;     // [RING]    consumers -> scheduler
  uint64_t* done = sempty + G_RING;      // [1]       all MMAs retired
  uint64_t* ep1 = done + 1;              // [1]       split tile: 4 epilogue warps wrote
  uint64_t* ep2 = ep1 + 1;               // [1]       split tile: arrival counted
  int* stile = (int*)(ep2 + 1);          // [RING]
  uint32_t* tmem_slot = (uint32_t*)(stile + G_RING);
  int* sflag = (int*)(tmem_slot + 1);    // split tile: units done before this one

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);
    }
    for (int r = 0; r < G_RING; ++r) {
      mbar_init(smem_u32(&sfull[r]), 1);
      mbar_init(smem_u32(&sempty[r]), 5);  // MMA thread + 4 epilogue warps
    }
    mbar_init(smem_u32(done), 1);
    mbar_init(smem_u32(ep1), 4);
    mbar_init(smem_u32(ep2), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * G_BN));
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
      const int c = (int)atomicAdd(args.counter, 1u);
      const int t = c < args.ntiles ? c : -1;
      const int slot = j % G_RING;
      ok = mbar_wait_bounded(smem_u32(&sempty[slot]), ((j / G_RING) & 1) ^ 1, args.status,
                             args.wait_ns);
      if (!ok) break;
      stile[slot] = t;
      mbar_arrive(smem_u32(&sfull[slot]));
      if (t < 0) break;
      const GTile T = args.tiles[t];
      if (T.nkb == 0) continue;
      const int nkb = T.nkb * KB_PER_PAD;
      if (args.work) atomicAdd(args.work, (double)nkb * (2.0 * G_BM * T.nw * BKE));
      const int nbox = (T.nw + G_BOXN - 1) / G_BOXN;
      const uint32_t bytes = (uint32_t)(A_BYTES + nbox * BOX_BYTES);
      for (int pair = 0; pair < 3 && ok; ++pair) {
        const int planeA = (pair == 2) ? 1 : 0, planeB = (pair == 1) ? 1 : 0;
        for (int kb = 0; kb < nkb; ++kb) {
          const int s = g % STAGES;
          ok = mbar_wait_bounded(smem_u32(&empty[s]), ((g / STAGES) & 1) ^ 1, args.status,
                                 args.wait_ns);
          if (!ok) break;
          const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t fb = smem_u32(&full[s]);
          mbar_expect_tx(fb, bytes);
          const int kx = (T.kb0 * KB_PER_PAD + kb) * BKE;
          tma_load_3d(sa, &mapA, fb, kx, T.m0, planeA);
          for (int i = 0; i < nbox; ++i)
            tma_load_3d(sa + A_BYTES + i * BOX_BYTES, &mapB, fb, kx, T.n0 + i * G_BOXN, planeB);
          ++g;
          ++issued;
        }
      }
    }
    if (!ok) {
      // drain the copies still in flight before this CTA may exit
      for (uint32_t it = issued > (uint32_t)STAGES ? issued - STAGES : 0; it < issued; ++it)
        mbar_wait_bounded(smem_u32(&full[it % STAGES]), (it / STAGES) & 1, args.status,
                          DRAIN_WAIT_NS);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    uint32_t g = 0, acc = 0;
    bool ok = true;
    for (int j = 0; ok; ++j) {
      const int slot = j % G_RING;
      ok = mbar_wait_bounded(smem_u32(&sfull[slot]), (j / G_RING) & 1, args.status,
                             args.wait_ns);
      if (!ok) break;
      const int t = stile[slot];
      mbar_arrive(smem_u32(&sempty[slot]));
      if (t < 0) break;
      const GTile T = args.tiles[t];
      if (T.nkb == 0) continue;
      const uint32_t buf = acc & 1;
      ok = mbar_wait_bounded(smem_u32(&tempty[buf]), ((acc >> 1) & 1) ^ 1, args.status,
                             args.wait_ns);
      if (!ok) break;
      tc_fence_after();
      const uint32_t d = tmem + buf * G_BN;
      const uint32_t idesc = TF32 ? idesc_tf32(G_BM, T.nw) : idesc_bf16(G_BM, T.nw);
      const int total = 3 * T.nkb * KB_PER_PAD;
      for (int it = 0; it < total; ++it) {
        const int s = g % STAGES;
        ok = mbar_wait_bounded(smem_u32(&full[s]), (g / STAGES) & 1, args.status, args.wait_ns);
        if (!ok) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
        const uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sa + A_BYTES);
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
    // ---------------- epilogue: TMEM -> registers -> C
    const int q = warp % 4;  // TMEM lane quarter accessible by this warp
    float* xb = xbuf + (warp - 2) * 32 * 33;
    const bool f32 = args.c_f32 != 0;
    const double alpha = args.alpha, beta = args.beta;
    const bool copy_f32 = f32 && alpha == 1.0 && beta == 0.0;
    const bool alpha_one = alpha == 1.0, beta_one = beta == 1.0;
    auto loadC = [&](int64_t e) -> double {
      return f32 ? (double)((const float*)args.C)[e] : ((const double*)args.C)[e];
    };
    auto putC = [&](int64_t e, double v) {
      if (f32) ((float*)args.C)[e] = (float)v;
      else ((double*)args.C)[e] = v;
    };
    uint32_t acc = 0, nsp = 0;
    for (int j = 0;; ++j) {
      const int slot = j % G_RING;
      bool ok = mbar_wait_bounded(smem_u32(&sfull[slot]), (j / G_RING) & 1, args.status,
                                  args.wait_ns);
      ok = __all_sync(0xffffffffu, ok);
      const int t = ok ? stile[slot] : -1;
      __syncwarp();
      if (ok && lane == 0) mbar_arrive(smem_u32(&sempty[slot]));
      if (t < 0) break;
      const GTile T = args.tiles[t];
      const int64_t mrow0 = (int64_t)T.m0 + 32 * q;  // first tile row of this warp
      const int64_t mr = mrow0 + lane;
      const bool rvalid = mr < T.mlim;
      const int64_t roff = rvalid ? args.rowoff[mr] : 0;
      const int64_t nend = std::min<int64_t>((int64_t)T.n0 + T.nw, T.nlim);
      // C (+)= alpha * v for 32 columns c0.. of this warp's 32 rows (v: lane = row); the
      // beta * C terms are all loaded before any store, so their latencies overlap
      auto store_chunk = [&](int c0, const uint32_t (&v)[32]) {
        const int64_t nl = (int64_t)T.n0 + c0 + lane;
        if (copy_f32 && !args.trans_store) {
          // FP32 output that is the accumulator itself: no FP64 arithmetic
          const int64_t myco = nl < nend ? args.coloff[nl] : 0;
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            const int64_t co = __shfl_sync(0xffffffffu, myco, jj);
            if (rvalid && (int64_t)T.n0 + c0 + jj < nend)
              ((float*)args.C)[roff + co] = __uint_as_float(v[jj]);
          }
          return;
        }
        if (!args.trans_store) {
          const int64_t myco = nl < nend ? args.coloff[nl] : 0;
#pragma unroll
          for (int h = 0; h < 32; h += 16) {  // two halves: fewer live registers
            int64_t co[16];
            double val[16];
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) {
              co[jj] = __shfl_sync(0xffffffffu, myco, h + jj);
              val[jj] = (double)__uint_as_float(v[h + jj]);
            }
            if (!alpha_one) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) val[jj] *= alpha;
            }
            if (beta != 0.0 && rvalid) {
              double cv[16];
#pragma unroll
              for (int jj = 0; jj < 16; ++jj)
                cv[jj] = ((int64_t)T.n0 + c0 + h + jj < nend) ? loadC(roff + co[jj]) : 0.0;
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) val[jj] = beta_one ? cv[jj] + val[jj] : fma(beta, cv[jj], val[jj]);
            }
            if (rvalid) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj)
                if ((int64_t)T.n0 + c0 + h + jj < nend) putC(roff + co[jj], val[jj]);
            }
          }
        } else {
          // transpose through shared memory: lane t then holds column c0 + t of the warp's
          // 32 rows, so that consecutive lanes store to consecutive addresses
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) xb[lane * 33 + jj] = __uint_as_float(v[jj]);
          __syncwarp();
          const bool cvalid = nl < nend;
          const int64_t co = cvalid ? args.coloff[nl] : 0;
          if (copy_f32) {
            // FP32 output that is the accumulator itself: no FP64 arithmetic or conversion.
            // All 32 values are read from shared memory before the first global store, so the
            // stores issue back to back.
            float fv[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) fv[i] = xb[i * 33 + lane];
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const int64_t r = __shfl_sync(0xffffffffu, roff, i);
              if (cvalid && mrow0 + i < T.mlim) ((float*)args.C)[r + co] = fv[i];
            }
            __syncwarp();
            return;
          }
#pragma unroll
          for (int h = 0; h < 32; h += 16) {
            int64_t ro[16];
            double val[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              ro[i] = __shfl_sync(0xffffffffu, roff, h + i);
              val[i] = (double)xb[(h + i) * 33 + lane];
            }
            if (!alpha_one) {
#pragma unroll
              for (int i = 0; i < 16; ++i) val[i] *= alpha;
            }
            if (beta != 0.0 && cvalid) {
              double cv[16];
#pragma unroll
              for (int i = 0; i < 16; ++i)
                cv[i] = (mrow0 + h + i < T.mlim) ? loadC(ro[i] + co) : 0.0;
#pragma unroll
              for (int i = 0; i < 16; ++i) val[i] = beta_one ? cv[i] + val[i] : fma(beta, cv[i], val[i]);
            }
            if (cvalid) {
#pragma unroll
              for (int i = 0; i < 16; ++i)
                if (mrow0 + h + i < T.mlim) putC(ro[i] + co, val[i]);
            }
          }
          __syncwarp();
        }
      };
      if (T.nkb == 0) {
        // no K member in this group: C = beta * C over the tile
        if (rvalid)
          for (int64_t n = T.n0; n < nend; ++n) {
            const int64_t e = roff + args.coloff[n];
            putC(e, beta != 0.0 ? beta * loadC(e) : 0.0);
          }
        continue;
      }
      const uint32_t buf = acc & 1;
      ok = mbar_wait_bounded(smem_u32(&tfull[buf]), (acc >> 1) & 1, args.status, args.wait_ns);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      tc_fence_after();
      if (T.nsplit > 1) {
        // split K: every unit writes its partial sums to its slot ([column][row], lane = row);
        // the last unit of the tile to finish adds all slots in unit order and stores
        float* own = args.partial + (size_t)(T.pslot + T.sid) * (G_BM * G_BN);
#pragma unroll 1
        for (int c0 = 0; c0 < T.nw; c0 += 32) {
          uint32_t v[32];
          const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * G_BN + (uint32_t)c0;
          TMEM_LD32(taddr, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int jj = 0; jj < 32; ++jj)
            own[(size_t)(c0 + jj) * G_BM + 32 * q + lane] = __uint_as_float(v[jj]);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&tempty[buf]));
        ++acc;
        __threadfence();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(ep1));
        if (warp == 2 && lane == 0) {
          bool w1 = mbar_wait_bounded(smem_u32(ep1), nsp & 1, args.status, args.wait_ns);
          int before = -1;
          if (w1) {
            before = (int)atomicAdd(&args.arrive[T.cslot], 1u);
            if (before == T.nsplit - 1) args.arrive[T.cslot] = 0;  // ready for the next launch
            __threadfence();
          }
          *sflag = before;
          mbar_arrive(smem_u32(ep2));
        }
        ok = mbar_wait_bounded(smem_u32(ep2), nsp & 1, args.status, args.wait_ns);
        ok = __all_sync(0xffffffffu, ok);
        ++nsp;
        if (!ok) break;
        const int before = *sflag;
        if (before < 0) break;  // the arrival wait ran out: status already recorded
        if (before != T.nsplit - 1) continue;
        __threadfence();
#pragma unroll 1
        for (int c0 = 0; c0 < T.nw; c0 += 32) {
          float sum[32];
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) sum[jj] = 0.0f;
          for (int u = 0; u < T.nsplit; ++u) {
            const float* pu = args.partial + (size_t)(T.pslot + u) * (G_BM * G_BN) +
                              (size_t)c0 * G_BM + 32 * q + lane;
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) sum[jj] += __ldcg(pu + (size_t)jj * G_BM);
          }
          uint32_t v[32];
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) v[jj] = __float_as_uint(sum[jj]);
          store_chunk(c0, v);
        }
        continue;
      }
#pragma unroll 1
      for (int c0 = 0; c0 < T.nw; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * G_BN + (uint32_t)c0;
        TMEM_LD32(taddr, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        store_chunk(c0, v);
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
                 "r"(2 * G_BN));
  }
}

void gemm_grouped(gb_ctx* ctx, const GPlan& p, const GOperand& A, const GOperand& B,
                  double alpha, double beta, void* C, bool c_f32) {
  GB_REQUIRE(tc_available(ctx), "grouped GEMM needs an sm_103 device");
  if (p.tiles.empty()) return;
  const GOperand& KA = p.trans ? B : A;
  const GOperand& KB = p.trans ? A : B;
  GB_REQUIRE(KA.kmax == p.kmax && KB.kmax == p.kmax && KA.esz == KB.esz,
             "grouped GEMM: operand packing mismatch");
  const bool tf32 = KA.esz == 4;
  CUtensorMap ma = make_plane_map(KA.data, KA.esz, KA.kmax, KA.rows, 2, G_BM);
  CUtensorMap mb = make_plane_map(KB.data, KB.esz, KB.kmax, KB.rows, 2, G_BOXN);
  GArgs a;
  a.tiles = p.d_tiles;
  a.ntiles = (int)p.tiles.size();
  // C is column-major: original rows (side 0) are adjacent in memory
  a.trans_store = p.trans ? 1 : 0;
  a.rowoff = p.d_rowoff;
  a.coloff = p.d_coloff;
  a.alpha = alpha;
  a.beta = beta;
  a.C = C;
  a.c_f32 = c_f32 ? 1 : 0;
  a.counter = ctx->d_tile_counter;
  a.status = ctx->d_status;
  a.wait_ns = ctx->wait_ns;
  a.work = (ctx->profiling || ctx->counting) ? ctx->d_work : nullptr;
  a.partial = p.d_partial;
  a.arrive = p.d_arrive;
  GB_REQUIRE(p.nslots == 0 || p.d_partial, "grouped GEMM: split-K buffers missing");
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
    ctx->prof_flops += p.block_flops;
    ctx->prof_kind.push_back(1);
    ctx->prof_kind_flops[1] += p.block_flops;
    GB_CHECK_CUDA(cudaEventRecord(ev0, ctx->stream));
  }
  GB_CHECK_CUDA(cudaMemsetAsync(ctx->d_tile_counter, 0, sizeof(unsigned int), ctx->stream));
  // split-K arrival counters start at zero whatever an earlier (possibly cut short) launch
  // left in them
  if (p.ncounters > 0)
    GB_CHECK_CUDA(cudaMemsetAsync(p.d_arrive, 0, (size_t)p.ncounters * sizeof(unsigned int),
                                  ctx->stream));
  const unsigned grid = (unsigned)std::min<int64_t>((int64_t)p.tiles.size(),
                                                    std::max(1, ctx->num_sms));
#define GB_GROUPED(ST_, TF_)                                                                  \
  do {                                                                                        \
    constexpr int SM = grouped_smem<ST_>();                                                   \
    static std::once_flag once;                                                               \
    std::call_once(once, [] {                                                                 \
      GB_CHECK_CUDA(cudaFuncSetAttribute(gemm_grouped_kernel<ST_, TF_>,                       \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SM));   \
    });                                                                                       \
    gemm_grouped_kernel<ST_, TF_><<<grid, G_THREADS, SM, ctx->stream>>>(ma, mb, a);           \
  } while (0)
  if (tf32) GB_GROUPED(4, true);
  else GB_GROUPED(4, false);
#undef GB_GROUPED
  GB_CHECK_CUDA(cudaGetLastError());
  if (ev1) GB_CHECK_CUDA(cudaEventRecord(ev1, ctx->stream));
  count_launch(ctx);
}

// ------------------------------------------------------------------ work counters
template <typename E>
__global__ void gcolcount_kernel(const E* __restrict__ hi, int64_t plane, int64_t kmax,
                                 const int32_t* __restrict__ gstart,
                                 const int32_t* __restrict__ klen, uint32_t* __restrict__ cnt) {
  const int g = blockIdx.y;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= klen[g]) return;
  const E* lo = hi + plane;
  uint32_t c = 0;
  for (int64_t r = gstart[g]; r < gstart[g + 1]; ++r)
    c += (plane_nz(hi[r * kmax + k]) || plane_nz(lo[r * kmax + k]));
  cnt[g * kmax + k] = c;
}

__global__ void gproducts_kernel(const uint32_t* __restrict__ ca, const uint32_t* __restrict__ cb,
                                 int64_t n, double* __restrict__ work) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)ca[i] * (double)cb[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(&work[1], 2.0 * acc);
}

void gcount_products(gb_ctx* ctx, const GPlan& p, const GOperand& A, const GOperand& B) {
  if (p.G == 0) return;
  const int64_t n = (int64_t)p.G * p.kmax;
  uint32_t* cnt = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(&cnt, 2 * n * sizeof(uint32_t), ctx->stream));
  GB_CHECK_CUDA(cudaMemsetAsync(cnt, 0, 2 * n * sizeof(uint32_t), ctx->stream));
  const GOperand* ops[2] = {&A, &B};
  for (int s = 0; s < 2; ++s) {
    const GOperand& o = *ops[s];
    dim3 grid((unsigned)((p.kmax + 255) / 256), (unsigned)p.G);
    if (o.esz == 4)
      gcolcount_kernel<float><<<grid, 256, 0, ctx->stream>>>(
          (const float*)o.data, o.rows * o.kmax, o.kmax, p.d_gstart[s], p.d_klen, cnt + s * n);
    else
      gcolcount_kernel<__nv_bfloat16><<<grid, 256, 0, ctx->stream>>>(
          (const __nv_bfloat16*)o.data, o.rows * o.kmax, o.kmax, p.d_gstart[s], p.d_klen,
          cnt + s * n);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
  }
  gproducts_kernel<<<64, 256, 0, ctx->stream>>>(cnt, cnt + n, n, ctx->d_work);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  GB_CHECK_CUDA(cudaFreeAsync(cnt, ctx->stream));
}

}  // namespace gb
