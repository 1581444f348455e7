// Shared runtime of libmpsgb: context, tensors, error state, scratch slots and the
// internal kernel entry points used by the operator, Krylov and gauge modules.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <functional>
#include <vector>

#include "../../include/mpsgb.h"

namespace gb {

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define GB_CHECK_CUDA(expr)                                                                 \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess)                                                                  \
      throw ::gb::Error(GB_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define GB_REQUIRE(cond, msg)                                  \
  do {                                                         \
    if (!(cond)) throw ::gb::Error(GB_ERR_ARG, std::string(msg)); \
  } while (0)

// ------------------------------------------------------------------ complex scalar
struct cplx {
  double re, im;
};

// ------------------------------------------------------------------ context / tensors
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};

enum ScratchSlot {
  SLOT_PACK_A = 0,
  SLOT_PACK_B,
  SLOT_T1,
  SLOT_T2,
  SLOT_RED,       // reduction partials
  SLOT_KRYLOV,    // Krylov basis
  SLOT_KRYLOV_W,  // Krylov work vector
  SLOT_GAUGE,     // factorisation buffers
  SLOT_GAUGE2,
  SLOT_GAUGE3,
  SLOT_TMP,       // short-lived helper buffers
  SLOT_TMP2,
  SLOT_SPLITK,    // split-K partial products of the FP64 GEMM
  SLOT_COUNT
};

struct LanePool;

}  // namespace gb

struct gb_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  int32_t* d_status = nullptr;   // device status word (bounded waits)
  // bound on every pipeline wait inside the tensor-core kernels (gb_ctx_set_wait_bound);
  // on expiry a kernel records GB_ERR_TIMEOUT, drains its copies and exits
  unsigned long long wait_ns = 2000000000ull;
  void* solver = nullptr;        // cusolverDnHandle_t
  void* solver_params = nullptr; // cusolverDnParams_t
  gb::Scratch scratch[gb::SLOT_COUNT];
  double* h_pinned = nullptr;    // small pinned host buffer for scalar readback
  size_t h_pinned_elems = 0;
  int num_sms = 0;
  bool lane = false;             // an auxiliary lane context (its GPU is shared with the others)
  int aux_prec = GB_PREC_FP64;   // precision of auxiliary state contractions
  int svd_method = 0;            // GB_SVD_* of gb_svd_trunc
  int eig_method = 0;            // GB_EIG_* of the Gram eigenproblems
  int lane_max = 8;              // host-thread lanes for per-sector work
  int staged_mix = 1;            // chain mix staged through shared memory: 0 never, 1 when
                                 // its rows have >= 4 entries on average, 2 always
  // split-precision GEMM schedule (GB_SCHED_*) and output tile width (0 = chosen per shape)
  int gemm_schedule = GB_SCHED_GROUPED;
  int gemm_bn = 0;
  unsigned int* d_tile_counter = nullptr;  // work counter of the persistent GEMM
  // work counters (device doubles): [0] flops the tensor pipe executes per split product
  // (tile granularity), [1] algorithmic flops of the nonzero products (block-sparse count)
  double* d_work = nullptr;
  bool counting = false;  // count nonzero products of every split GEMM (extra passes)
  // auxiliary contexts (own stream, scratch and solver handle) for many small independent
  // work items, e.g. the charge sectors of a U(1) factorisation (see run_on_lanes)
  std::vector<gb_ctx*> lanes;
  gb::LanePool* lane_pool = nullptr;  // persistent host threads driving the lanes
  // tracing of the tensor-core GEMM launches
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;  // pairs (start, stop) per launch
  size_t prof_used = 0;
  double prof_flops = 0.0;
  // per kernel family (0: dense-embedding split GEMM, 1: grouped sector-block GEMM): the
  // family of every event pair, the flops issued, and after profile_end the summed results
  std::vector<int> prof_kind;
  double prof_kind_flops[2] = {0.0, 0.0};
  double prof_res_ms[2] = {0.0, 0.0};
  int64_t prof_res_n[2] = {0, 0};
  double prof_res_flops[2] = {0.0, 0.0};
  cudaEvent_t prof_region[2] = {nullptr, nullptr};
  // launch trace: an event after every counted launch (and every trace point), tagged with
  // the source site that issued it; the time between consecutive events is charged to the
  // later site (its kernel plus any idle gap before it)
  bool tracing = false;
  std::vector<cudaEvent_t> trace_ev;
  std::vector<int> trace_site;
  size_t trace_used = 0;
  cudaEvent_t trace_start = nullptr;
  std::vector<int> trace_res_site;  // per site after gb_ctx_trace_end: id, ms, launches
  std::vector<double> trace_res_ms;
  std::vector<int64_t> trace_res_n;
};

struct gb_tensor {
  gb_ctx* ctx = nullptr;
  int kind = GB_KIND_GENERIC;
  int dtype = GB_F64;
  int ndim = 0;
  int64_t dims[6] = {0, 0, 0, 0, 0, 0};  // reference leg order
  void* data = nullptr;                  // device pointer, device layout
  size_t bytes = 0;
  std::vector<double> host_mpo;          // host mirror for GB_KIND_MPO (interleaved if complex)
};

namespace gb {

inline size_t elem_size(int dtype) { return dtype == GB_C128 ? 16 : 8; }
inline int64_t numel(const gb_tensor* t) {
  int64_t n = 1;
  for (int i = 0; i < t->ndim; ++i) n *= t->dims[i];
  return n;
}
inline bool is_cplx(int dtype) { return dtype == GB_C128; }

void* scratch(gb_ctx* ctx, int slot, size_t bytes);
// fn(lane, i) for i < n on up to 8 lane contexts, one host thread per lane: the parent's
// stream is synchronised first, every lane's stream at the end; the first exception thrown
// by any item is rethrown after all lanes stopped
// (run_on_lanes: the launch trace charges the lanes' work to the calling source line)
void run_on_lanes_at(gb_ctx* ctx, int64_t n, const char* file, int line,
                     const std::function<void(gb_ctx*, int64_t)>& fn);
#define run_on_lanes(ctx, n, ...) \
  ::gb::run_on_lanes_at((ctx), (n), __FILE__, __LINE__, __VA_ARGS__)
// U(1) operators (after gb_heff_set_sectors): the Krylov solvers keep only the n allowed
// entries of their vectors; xcomp is an operator-owned compact vector
struct HeffCompact {
  int64_t n = 0;
  void* xcomp = nullptr;
};
bool heff_compact(gb_heff* h, HeffCompact* c);
void heff_gather(gb_heff* h, const void* dense, void* compact);
void heff_scatter(gb_heff* h, const void* compact, void* dense);  // zero-fills dense first
void heff_apply_compact(gb_heff* h, const void* x, void* y);

// launch accounting (and, while tracing, an event tagged with the issuing source line)
void trace_point(gb_ctx* ctx, const char* file, int line);
inline void count_launch_at(gb_ctx* ctx, int n, const char* file, int line) {
  ctx->launches += n;
  if (ctx->tracing) trace_point(ctx, file, line);
}
#define count_launch(ctx) ::gb::count_launch_at((ctx), 1, __FILE__, __LINE__)
#define count_launch_n(ctx, n) ::gb::count_launch_at((ctx), (n), __FILE__, __LINE__)
// a trace point after work that is not a counted kernel (library calls, copies)
#define GB_TRACE(ctx) \
  do {                                                             \
    if ((ctx)->tracing) ::gb::trace_point((ctx), __FILE__, __LINE__); \
  } while (0)

// ------------------------------------------------------------------ kernel launchers
// All operate on ctx->stream and count their launches.

// General strided permute/copy: out[o] = in[i] over up to 6 dims.
// dims/out_strides/in_strides are element strides for each logical dim.
void permute(gb_ctx* ctx, int dtype, int nd, const int64_t* dims, const void* in,
             const int64_t* in_strides, void* out, const int64_t* out_strides);

// Sparse mode mix (see kernels.cu):
// y[a*ya + out_off[J] + n*yn] = beta*y + sum_{e in row J} val[e] * x[a*xa + in_off[col[e]] + n*xn]
struct MixPlan {
  int64_t A = 1, N = 1, nI = 0, nJ = 0;
  int64_t xa = 1, xn = 0, ya = 1, yn = 0;
  std::vector<int64_t> in_off, out_off;
  std::vector<int> row_ptr, col;
  std::vector<double> val;  // interleaved (re, im) when complex
  bool cplx = false;
};
struct MixDev {
  void* buf = nullptr;  // device copy of tables
  size_t bytes = 0;
  int64_t A = 1, N = 1, nJ = 0, xa = 1, xn = 0, ya = 1, yn = 0;
  bool cplx = false;
  const int64_t* in_off = nullptr;
  const int64_t* out_off = nullptr;
  const int* row_ptr = nullptr;
  const int* col = nullptr;
  const double* val = nullptr;
};
MixDev mix_upload(gb_ctx* ctx, const MixPlan& p);
void mix_free(MixDev& m);
void mix_run(gb_ctx* ctx, const MixDev& m, int dtype, const void* x, void* y, double beta);

// y[off_J + i*ds] += val_J for i < count (diagonal additions of delta terms)
void add_diag(gb_ctx* ctx, int dtype, void* y, const std::vector<int64_t>& offs,
              const std::vector<double>& vals, int64_t count, int64_t ds);

// FP64 / complex GEMM on CUDA cores, column-major, batched with strides.
// op: 'N', 'T' or 'C'.  C = alpha*op(A)*op(B) + beta*C (beta = 0 does not read C).
void gemm_fp64(gb_ctx* ctx, int dtype, char opA, char opB, int64_t M, int64_t N, int64_t K,
               cplx alpha, const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb,
               int64_t sB, cplx beta, void* C, int64_t ldc, int64_t sC, int64_t batch);

// BLAS-1 style helpers over n elements of dtype
void fill_zero(gb_ctx* ctx, void* p, size_t bytes);
void axpy(gb_ctx* ctx, int dtype, int64_t n, cplx a, const void* x, void* y);
void scale(gb_ctx* ctx, int dtype, int64_t n, cplx a, void* x);
cplx dot(gb_ctx* ctx, int dtype, int64_t n, const void* x, const void* y);  // conj(x).y
double nrm2(gb_ctx* ctx, int dtype, int64_t n, const void* x);
// c[j] = sum_i conj(V[i + ld*j]) w[i] for j < k; result copied to host (k values)
void multi_dot(gb_ctx* ctx, int dtype, int64_t n, int k, const void* V, int64_t ld,
               const void* w, cplx* host_out);
// w[i] += sum_j V[i + ld*j] * coef[j] for j < k (coef from host)
void multi_axpy(gb_ctx* ctx, int dtype, int64_t n, int k, const void* V, int64_t ld,
                const cplx* coef, void* w);
// finite check: returns true when all entries are finite
bool all_finite(gb_ctx* ctx, int dtype, int64_t n, const void* x);

// ------------------------------------------------------------------ split precision
// Operand packed for the tcgen05 BF16 GEMM: K-major rows, two planes (hi, lo),
// realified when complex (see gemm_tc.cu).
//
// Each packed operand carries a nonzero map: one bit per (128-row tile, 64-wide k-block),
// [batch][ceil(rows/128)][kw] 32-bit words stored after the planes.  A bit is set when any
// entry of that tile is nonzero; the persistent GEMM skips k-blocks whose A and B bits are
// not both set, which is how block-sparse (charge-conserving) operands stored densely with
// charge-sorted legs run only their nonzero blocks.
constexpr int64_t MASK_ROWS = 128;
struct Packed {
  void* data = nullptr;  // [batch][2 planes][rows][Kp] bf16
  int64_t rows = 0, Kp = 0, batch = 1;
  int64_t K = 0;         // logical K (per real/imag half when complex)
  int64_t Kh = 0;        // offset of the imaginary half along K when complex
  bool cplx = false;
  bool owned = false;
  size_t bytes = 0;
  uint32_t* mask = nullptr;  // nonzero map (see above)
  int64_t mrows = 0;         // ceil(rows / 128)
  int kw = 0;                // 32-bit words per mask row: ceil(Kp / 64 / 32)
  uint32_t* cnt = nullptr;   // [batch][Kp] nonzero rows per packed k (filled when counting)
  bool cnt_valid = false;
  int esz = 2;               // plane element bytes: 2 (BF16 planes) or 4 (TF32 planes)
  int bk = 64;               // k-block (elements per 128-byte swizzle row): 64 or 32
};
// which operand of C = op(A) op(B) is being packed
enum PackRole { PACK_AS_A = 0, PACK_AS_B = 1 };
// prec: GB_PREC_BF16X3 (BF16 planes) or GB_PREC_TF32X3 (TF32 planes in 32-bit words)
size_t packed_bytes(int64_t rows, int64_t K, bool cplx, int role, int64_t batch,
                    int prec = GB_PREC_BF16X3);
// fills every field of out for a buffer of packed_bytes(...) at data
void packed_layout(Packed& out, void* data, int64_t R, int64_t K, bool cplx, int role,
                   int64_t batch, int prec = GB_PREC_BF16X3);
void pack_operand(gb_ctx* ctx, int dtype, int role, char op, int64_t M_or_N, int64_t K,
                  const void* src, int64_t ld, int64_t stride, int64_t batch, Packed& out,
                  void* dst, int prec = GB_PREC_BF16X3);
// Skipping structurally zero work in mixpack_run: x is the output of a GEMM with an output
// map (xmap, onc columns of 128 per row tile of 128); input i of the mix at (a, n) sits at
// row a + roff[i], column coff[i] + n*xnM of that matrix.  prev: scratch of the packed
// output's map size that receives the previous map (the planes must have been zeroed when
// allocated, and the K padding is then never touched again).
struct MixSkipDev {
  const uint32_t* xmap = nullptr;
  int64_t onc = 0;
  const int64_t* roff = nullptr;
  const int64_t* coff = nullptr;
  int64_t xnM = 0;
  uint32_t* prev = nullptr;
  // U(1) sectors (optional): output (a, J, n) is structurally zero outside
  // a in [arange[J + nJ*n].x, .y); those entries are never written (they stay zero)
  const int2* arange = nullptr;
  int64_t arange_max = 0;
};
// leg mix whose output is written directly as the packed B operand of the next GEMM
// (kJ[J]: contraction-index offset of output row J, mJ[J] + n*mn: output column index)
void mixpack_run(gb_ctx* ctx, const MixDev& m, const int64_t* kJ, const int64_t* mJ, int64_t mn,
                 int dtype, const void* x, Packed& out, int64_t Klog, int64_t Nlog,
                 const MixSkipDev* skip = nullptr, bool x_f32 = false);
// outmap (optional, batch 1, split precision only): bit (m/128)*ceil(N/128) + n/128 is set
// for every 128 x 128 region of C that receives a contribution.  For real data the regions
// that receive none are not written, except where the previous call with the same map wrote
// them: those are overwritten with zeros.  The buffer holds two maps (2 * outmap_bytes): the
// current one and, behind it, the previous call's; started at zero together with C, every
// region outside the current map then holds zeros.
size_t outmap_bytes(int64_t M, int64_t N);
// c_f32: C is stored in FP32 (exact for alpha = 1, beta = 0: the FP32 accumulator itself)
void gemm_split(gb_ctx* ctx, int dtype, const Packed& A, const Packed& B, int64_t M,
                int64_t N, double alpha, double beta, void* C, int64_t ldc, int64_t sC,
                uint32_t* outmap = nullptr, bool c_f32 = false);
bool tc_available(gb_ctx* ctx);

// tile-packed copies of block-sparse tensors (packed.cu)
gb_packed* tensor_pack(gb_ctx* ctx, const gb_tensor* t);
void packed_unpack(gb_ctx* ctx, const gb_packed* p, gb_tensor* out);
void packed_info(const gb_packed* p, int64_t* kept, int64_t* total, size_t* bytes);
gb_ctx* packed_ctx(const gb_packed* p);
void packed_free(gb_packed* p);

// Hermitian eigendecomposition of the g x g matrix G in place (eigenvectors overwrite G,
// eigenvalues ascending in W), by the context's GB_EIG_* method; *info (device) is nonzero on
// failure.  Synchronises the context's stream before returning.
void sym_eig(gb_ctx* ctx, int dtype, int64_t g, void* G, double* W, int* info);

// Unified GEMM: dispatches on precision; optional pre-packed operands.
void gemm(gb_ctx* ctx, int prec, int dtype, char opA, char opB, int64_t M, int64_t N,
          int64_t K, double alpha, const void* A, int64_t lda, int64_t sA, const void* B,
          int64_t ldb, int64_t sB, double beta, void* C, int64_t ldc, int64_t sC,
          int64_t batch = 1, const Packed* pA = nullptr, const Packed* pB = nullptr,
          uint32_t* outmap = nullptr, bool c_f32 = false);

}  // namespace gb
