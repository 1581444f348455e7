// Grouped split-precision GEMM over U(1) sector blocks (see grouped.cu).
//
// A contraction C[M x N] (+)= A[M x K] B[K x N] between charge-conserving tensors is
// block diagonal once every index carries its charge label: A[m, k] != 0 only if
// label(m) = label(k), B[k, n] != 0 only if label(k) = label(n).  The plan lists the
// labels present on all sides ("groups"); every operand is packed block-stacked -- group g
// occupies its own rows of a K-major plane pair, with its K members in columns
// [0, kpad_g) -- and the persistent tcgen05 kernel runs only the tiles of the diagonal
// blocks, with per-tile MMA width, writing each element back to its place in the
// charge-sorted dense embedding through per-row / per-column offsets.
#pragma once

#include <climits>
#include <vector>

#include "gb_common.h"

namespace gb {

// charge sources of a leg: which charge array labels it
enum LegCharge { Q_NONE = 0, Q_L, Q_R, Q_P1, Q_P2, Q_CL, Q_CR, Q_COUNT };
struct LegSpec {
  int64_t n = 1;     // extent
  int which = Q_NONE;
  int sign = 1;      // contribution of the leg's charge to the label
};
constexpr int32_t NO_LABEL = INT32_MIN;  // index outside every group (an all-zero channel)

// labels of the mixed-radix index space of `legs` (first leg fastest); q[which] are the
// charge arrays (nullptr entries read as zero charges); a channel charge of NO_LABEL makes
// the whole index NO_LABEL
std::vector<int32_t> leg_labels(const std::vector<LegSpec>& legs,
                                const std::vector<const int32_t*>& q);

struct GTile {
  int32_t m0, n0;      // first packed row of the tile in the kernel's A / B row space
  int32_t nkb;         // K blocks of this work unit (0: the tile only writes beta * C)
  int32_t nw;          // MMA N of the tile (multiple of 16, <= 256)
  int32_t mlim, nlim;  // end of the tile's group in the A / B row space (exclusive)
  int32_t g;
  int32_t kb0;         // first K block of the unit within its group
  int32_t nsplit;      // units sharing the output tile (split K); 1: the whole K
  int32_t sid;         // index of this unit among them
  int32_t pslot;       // partial-sum slot of unit 0 of the tile (unit sid uses pslot + sid)
  int32_t cslot;       // arrival counter of the tile
};

struct GPackTile {
  int32_t rp0, nr, g, kp0;  // 32-row x 32-column block of group g
};

// block-stacked split planes: [2][rows][kmax] (hi, lo), group g in rows
// [gstart[g], gstart[g + 1]), its K members in columns [0, kpad[g]) (zeros beyond klen[g])
struct GOperand {
  void* data = nullptr;
  int64_t rows = 0, kmax = 0;
  int esz = 2;
  size_t bytes = 0;
};

// one side of the plan: the packed row space of the M (or N) index of the GEMM
struct GSide {
  std::vector<int32_t> dense;   // packed row -> dense index
  std::vector<int32_t> gstart;  // group g: rows [gstart[g], gstart[g + 1])
  std::vector<GPackTile> ptiles;
  int64_t rows_alloc = 0;       // packed rows rounded up to 128
};

struct GPlan {
  int G = 0;
  std::vector<int32_t> label;
  GSide side[2];                // [0] = M (rows of the original A), [1] = N (original B)
  std::vector<int32_t> kdense;  // group K members (dense k), concatenated
  std::vector<int32_t> kstart;  // group g: kdense[kstart[g] .. kstart[g + 1])
  std::vector<int32_t> kpad;    // group g: padded K (multiple of 64)
  int64_t kmax = 64;
  bool trans = false;           // the kernel's A is the original B (M and N swapped)
  int64_t ldc = 0;              // leading dimension of the column-major output
  std::vector<GTile> tiles;
  double tile_flops = 0.0;      // tensor-pipe flops per split product (BF16 K-block count)
  double block_flops = 0.0;     // 2 sum_g M_g N_g K_g
  int nslots = 0;               // partial-sum slots of the split-K units
  int ncounters = 0;            // output tiles computed by more than one unit
  // device copies (one owned buffer)
  void* dev = nullptr;
  GTile* d_tiles = nullptr;
  int64_t* d_rowoff = nullptr;  // kernel A-row -> output offset
  int64_t* d_coloff = nullptr;  // kernel B-row -> output offset
  int32_t* d_dense[2] = {nullptr, nullptr};
  int32_t* d_gstart[2] = {nullptr, nullptr};
  GPackTile* d_ptiles[2] = {nullptr, nullptr};
  int32_t* d_kdense = nullptr;
  int32_t* d_kstart = nullptr;
  int32_t* d_klen = nullptr;
  float* d_partial = nullptr;       // [nslots][G_BN columns][128 rows] FP32 partial sums
  unsigned int* d_arrive = nullptr; // [ncounters] units of a split tile done (reset to 0)
};

// Plan of C = A B with dense labels of M, K, N.  first_writer: the GEMM overwrites C
// (beta = 0), so groups without K members still get tiles that write zeros.  ldc: leading
// dimension of the column-major output (element offsets).
// sms: multiprocessors of the device; a tile whose K is long against the plan's total work
// per multiprocessor is split along K into units summed deterministically (in unit order)
// by the last of them to finish.
void gplan_build(GPlan& p, const std::vector<int32_t>& labM, const std::vector<int32_t>& labK,
                 const std::vector<int32_t>& labN, bool first_writer, int64_t ldc,
                 int sms = 152);
// device buffers of the plan (allocated through alloc, one call)
void gplan_upload(gb_ctx* ctx, GPlan& p, const std::function<void*(size_t)>& alloc);
size_t goperand_bytes(const GPlan& p, int side, int prec);
void goperand_init(gb_ctx* ctx, GOperand& op, const GPlan& p, int side, void* data, int prec);
// pack the original operand of `side` from a dense FP64 matrix: element (row r, k) of the
// operand at src[r * rs + k * ks]; returns the nonzero count of the packed blocks when
// count_nnz is set (synchronises), else 0.  With a range [klo, khi) of the plan's dense K
// index only those K members are packed, from src[r * rs + (k - klo) * ks], and nothing else
// of the operand is written: two sources stacked along K (a merged GEMM) pack separately.
int64_t gpack(gb_ctx* ctx, const GPlan& p, int side, const double* src, int64_t rs, int64_t ks,
              GOperand& op, bool count_nnz = false, int64_t klo = 0,
              int64_t khi = INT64_MAX);
// nonzero count of a dense column-major FP64 matrix rows x cols (leading dimension ld)
int64_t dense_nnz(gb_ctx* ctx, const double* src, int64_t rows, int64_t cols, int64_t ld);
// nonzero entries (r, k) of an operand (element at src[r * rs + k * ks]) whose labels
// labR[r] and labK[k] differ or are undefined: the entries the grouped form would drop
int64_t label_violations(gb_ctx* ctx, const double* src, int64_t R, int64_t K, int64_t rs,
                         int64_t ks, const std::vector<int32_t>& labR,
                         const std::vector<int32_t>& labK);

// the AA-chain mix written as a block-stacked operand: entry (J, n) covers the input rows
// a in [lo, hi), writes packed row `row`, columns kst + (a - lo)
struct GMixEntry {
  int32_t lo, hi, row, kst;
};
void gmix_run(gb_ctx* ctx, const MixDev& m, const GMixEntry* ent, int64_t span_max,
              const float* t1, GOperand& out);
// The same mix staged through shared memory.  The output rows J fall into groups whose
// input range [lo, hi) is the same at every column n (rows of one charge); a block per
// (column, group) loads the group's rows (local CSR) and the inputs they read -- once,
// coalesced -- into shared memory and computes every row of the group from there, four
// columns per thread.  The sums run over each row's entries in the order of gmix_run: the
// results are identical.
struct GMixStaged {
  int NL = 0;              // row groups
  double nnz_per_row = 0;  // mix entries per output row (the staged form pays off when dense)
  int chunk = 0;           // input rows a staged per pass (BF16 planes)
  int chunk_tf32 = 0;      // (TF32 planes: the coefficients' lo halves are staged too)
  int csr_floats = 0;      // shared-memory words of the largest group's rows
  int csr_floats_tf32 = 0;
  size_t smem = 0;         // dynamic shared memory per block
  size_t smem_tf32 = 0;
  const int2* rng = nullptr;    // [N][NL]: (lo, hi) of group g at column n
  const int* jlist = nullptr;   // rows of group g: jlist[jstart[g] .. jstart[g + 1])
  const int* jstart = nullptr;
  const int* ilist = nullptr;   // inputs read by group g: ilist[istart[g] .. istart[g + 1])
  const int* istart = nullptr;
  const int* rp = nullptr;      // row pointers of group g at rp[rstart[g]] (nj_g + 1 entries)
  const int* rstart = nullptr;
  const int* li = nullptr;      // entries of group g at [cstart[g], cstart[g + 1]): local
  const float* vh = nullptr;    // input index and coefficient as hi + lo floats
  const float* vl = nullptr;
  const int* cstart = nullptr;
};
void gmix_staged_run(gb_ctx* ctx, const MixDev& m, const GMixStaged& g, const GMixEntry* ent,
                     const float* t1, GOperand& out);

// C = alpha * (A B) + beta * C over the plan's tiles; c_f32: C holds FP32
void gemm_grouped(gb_ctx* ctx, const GPlan& p, const GOperand& A, const GOperand& B,
                  double alpha, double beta, void* C, bool c_f32);
// work counters (counting mode): nonzero products sum_g sum_k nnzA_g(k) nnzB_g(k)
void gcount_products(gb_ctx* ctx, const GPlan& p, const GOperand& A, const GOperand& B);

}  // namespace gb
