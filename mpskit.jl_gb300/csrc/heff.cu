// Effective local operators on the device.
//
// Build follows MPSKit's Jordan-form construction and `prepare_operator!!` folding
// (src/algorithms/derivatives/hamiltonian_derivatives.jl:44-157, 272-468): the cheap
// terms (II, ID, CB, DE, EE / D, I, E) are folded into the GEMM-shaped terms
// (IC, BE, CA, AB / C, B) exactly as the reference decides, and every term tensor is
// produced directly in the layout its GEMM consumes, by one sparse channel-combination
// pass over GL or GR (plus a diagonal pass for the delta-function terms).
//
// Apply is a short list of steps (GEMMs and sparse leg mixes) over the device layouts
//   x_AC2 (l, s1, s2, r), x_AC (l, s, r), x_C (l, r), GL (a, a', w), GR (b', w, b),
// chosen so that every term is a plain column-major GEMM on a view of x without any
// permutation.  The continuing-continuing term (AA / A) is evaluated as
//   T1 = x . GR_c ; T2 = (W1 W2)-mix(T1) ; y += GL_c . T2
// which is the same linear map as the reference's prepared L.x.R form with fewer
// flops (2 chi d^2 D^3 instead of 2 chi d^3 D^3 for AC2).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <sstream>

#include "gb_common.h"
#include "grouped.h"

using gb::cplx;
using gb::MixDev;
using gb::MixPlan;
using gb::Packed;

namespace {

enum Src { S_CONST = 0, S_X = 1, S_Y = 2, S_T1 = 3, S_T2 = 4 };

struct Step {
  bool is_gemm = true;
  // GEMM: dst = alpha * op(A) * op(B) + beta * dst
  int srcA = S_CONST, srcB = S_CONST, dst = S_Y;
  const void* cA = nullptr;
  const void* cB = nullptr;
  int64_t lda = 0, ldb = 0, ldc = 0;
  int64_t M = 0, N = 0, K = 0;
  char opA = 'N', opB = 'N';
  bool accumulate = true;  // beta = 1 (else 0)
  Packed pA, pB;           // pre-packed constant operands (split precision)
  bool hasPA = false, hasPB = false;
  // MIX: dst (+)= mix(src)
  int src = S_X;
  MixDev mix;
  MixPlan mixh;  // host copy of the plan (the chain mix only: its staged grouped form)
  std::string name;
  // the continuing-channel chain: the middle mix produces T2, the next GEMM consumes it;
  // in split precision the mix writes T2 directly as that GEMM's packed B operand
  bool t2_producer = false;
  bool t2_consumer = false;
  // U(1) labels of the GEMM's index spaces (M, K, N) for the grouped sector-block GEMM:
  // legs in the order of the dense index (first fastest)
  std::vector<gb::LegSpec> lM, lK, lN;
};

// grouped sector-block form of one GEMM step (after gb_heff_set_sectors)
struct GStep {
  gb::GPlan plan;
  gb::GOperand op[2];  // packed original A (side 0) and B (side 1)
};

struct Cx {
  double re = 0, im = 0;
};

// host copy of an MPO tensor W[wl, s, s', wr] (column-major) with value access
struct HostW {
  int64_t wl, d1, d2, wr;
  bool cplx;
  const std::vector<double>* v;
  Cx at(int64_t a, int64_t s, int64_t t, int64_t b) const {
    int64_t i = a + wl * (s + d1 * (t + d2 * b));
    if (cplx) return Cx{(*v)[2 * i], (*v)[2 * i + 1]};
    return Cx{(*v)[i], 0.0};
  }
  bool nz(int64_t a, int64_t s, int64_t t, int64_t b) const {
    Cx c = at(a, s, t, b);
    return c.re != 0.0 || c.im != 0.0;
  }
};

inline Cx cmul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx cadd(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }

// dense coefficient table coef[J][I] -> sparse mix plan
struct Coef {
  int64_t nJ, nI;
  std::vector<Cx> c;
  Coef(int64_t nj, int64_t ni) : nJ(nj), nI(ni), c(nj * ni) {}
  Cx& at(int64_t J, int64_t I) { return c[J * nI + I]; }
};

MixPlan make_plan(const Coef& cf, bool cx, int64_t A, int64_t N, int64_t xa, int64_t xn,
                  int64_t ya, int64_t yn, const std::vector<int64_t>& in_off,
                  const std::vector<int64_t>& out_off) {
  MixPlan p;
  p.A = A;
  p.N = N;
  p.xa = xa;
  p.xn = xn;
  p.ya = ya;
  p.yn = yn;
  p.nI = cf.nI;
  p.nJ = cf.nJ;
  p.in_off = in_off;
  p.out_off = out_off;
  p.cplx = cx;
  p.row_ptr.push_back(0);
  for (int64_t J = 0; J < cf.nJ; ++J) {
    for (int64_t I = 0; I < cf.nI; ++I) {
      Cx v = cf.c[J * cf.nI + I];
      if (v.re == 0.0 && v.im == 0.0) continue;
      p.col.push_back((int)I);
      p.val.push_back(v.re);
      if (cx) p.val.push_back(v.im);
    }
    p.row_ptr.push_back((int)p.col.size());
  }
  return p;
}

}  // namespace

struct gb_heff {
  gb_ctx* ctx = nullptr;
  int kind = 0, dtype = GB_F64, prec = GB_PREC_FP64;
  int64_t xdims[4] = {0, 0, 0, 0};  // reference dims of x
  int xndim = 0;
  int64_t xnumel = 0;
  std::vector<Step> steps;
  std::vector<void*> owned;           // device buffers owned by the operator
  int64_t t1_elems = 0, t2_elems = 0;
  double flops = 0.0;
  std::string terms;
  bool y_zero_first = false;  // y must be zeroed before the steps (no step overwrites it)
  void* t1 = nullptr;
  void* t2 = nullptr;
  // packed-T2 path (split precision): output-row offsets of the mix in the packed B operand
  std::vector<int64_t> kJ, mJ;
  int64_t mn = 0, t2K = 0, t2N = 0;
  void* kmJ_dev = nullptr;
  Packed t2p;
  bool t2p_ready = false;
  // structurally zero regions of the AA chain (split precision): the T1 GEMM records which
  // 128 x 128 regions of T1 it wrote (t1map), and the fused mix reads only those; input i
  // of the mix at (a, n) is T1[a + t1roff[i], t1coff[i] + n * t1xnM]
  int64_t t1M = 0, t1N = 0, t1xnM = 0;
  std::vector<int64_t> t1roff, t1coff;
  uint32_t* t1map = nullptr;
  int64_t* t1rc_dev = nullptr;
  uint32_t* t2prev = nullptr;
  bool t1_f32 = false;  // T1 currently holds FP32 values (fused split chain)
  // U(1) sectors of the fused chain (gb_heff_set_sectors): output row J of the mix is
  // (continuing channel Jc[J], fused physical index Jp[J]); element (a, J, n) may be nonzero
  // only for a in arange[J + nJ * n] -- the l' sector of charge q_r(n) - dq_c - q_p
  const void* aa_glc = nullptr;  // GL's continuing channels (l, l', c)
  int64_t aa_chr = 0, aa_Dl = 0, aa_Dr = 0, aa_np = 0;
  std::vector<int64_t> Jc, Jp;
  int2* arange = nullptr;
  int64_t arange_max = 0;
  // U(1) sectors of x itself: column j of the device layout (l fastest) holds its allowed
  // entries in one run of l; runs[3j..3j+2] = (compact offset, dense offset, length)
  int64_t* runs = nullptr;
  int64_t nruns = 0, ncompact = 0;
  void* xfull = nullptr;  // dense staging of the Krylov solvers (zero outside the runs)
  void* yfull = nullptr;
  void* xcomp = nullptr;  // a compact state vector (exponentiate)
  // grouped sector-block GEMMs (GB_SCHED_GROUPED, split precision, real data): one plan per
  // GEMM step, the AA-chain mix written straight into the block-stacked T2 operand
  int sched = 0;                 // GEMM schedule of the context at build time
  const void* aa_grc = nullptr;  // GR's continuing channels (r', j, r)
  int64_t aa_chc = 0;
  std::vector<int32_t> q_l, q_r, q_p1, q_p2, dq_l, dq_r;  // charges (host)
  std::vector<int2> arange_h;    // host copy of arange
  std::vector<GStep> gsteps;     // index-aligned with steps
  // a step whose GEMM runs inside another's (the constant-x term CA / C stacked along K
  // onto the chain's last GEMM, same output blocks): merged_into[i] = that step, else -1;
  // merged_k[j] = K of step j's own part when step j carries a merged step
  std::vector<int> merged_into;
  std::vector<int64_t> merged_k;
  gb::GMixEntry* gmix = nullptr;
  gb::GMixStaged gmix_st;        // staged form of the same mix (gmix_st.NL > 0 when built)
  std::vector<int64_t> lam_J;    // charge of every chain row J (INT64_MIN: channel absent)
  int t2_step = -1;              // the step that consumes T2
  bool gp_ready = false;
  bool prepacked = false;        // constants of the dense-embedding path packed
  int gp_prec = -1;
};

namespace gb {

static void* dalloc(gb_heff* h, size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  // stream-ordered pool: operator buffers are recycled across local updates without
  // the device-wide synchronisation of cudaMalloc/cudaFree
  cudaError_t e = cudaMallocAsync(&p, bytes, h->ctx->stream);
  if (e != cudaSuccess) throw Error(GB_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->owned.push_back(p);
  return p;
}

// T1 is an M x N column-major matrix; the mix input i starts at offset io[i] and advances
// by M * xnM per output column n
static void record_t1_geometry(gb_heff* h, int64_t M, int64_t N, const std::vector<int64_t>& io,
                               int64_t xnM) {
  h->t1M = M;
  h->t1N = N;
  h->t1xnM = xnM;
  h->t1roff.resize(io.size());
  h->t1coff.resize(io.size());
  for (size_t i = 0; i < io.size(); ++i) {
    h->t1roff[i] = io[i] % M;
    h->t1coff[i] = io[i] / M;
  }
}

static void add_gemm_flops(gb_heff* h, const Step& s) {
  h->flops += (is_cplx(h->dtype) ? 8.0 : 2.0) * (double)s.M * (double)s.N * (double)s.K;
}

// Pre-pack constant GEMM operands for the split path.
static void prepare_t2p(gb_heff* h) {
  if (h->prec == GB_PREC_FP64 || h->t2p_ready || h->kJ.empty()) return;
  const bool cx = is_cplx(h->dtype);
  size_t nJ = h->kJ.size();
  h->kmJ_dev = dalloc(h, 2 * nJ * sizeof(int64_t));
  std::vector<int64_t> tab(h->kJ);
  tab.insert(tab.end(), h->mJ.begin(), h->mJ.end());
  GB_CHECK_CUDA(cudaMemcpyAsync(h->kmJ_dev, tab.data(), tab.size() * sizeof(int64_t),
                                cudaMemcpyHostToDevice, h->ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(h->ctx->stream));
  size_t bytes = packed_bytes(h->t2N, h->t2K, cx, PACK_AS_B, 1, h->prec);
  packed_layout(h->t2p, dalloc(h, bytes), h->t2N, h->t2K, cx, PACK_AS_B, 1, h->prec);
  // zeroed once: the fused mix then writes only entries that may be nonzero (see MixSkipDev)
  GB_CHECK_CUDA(cudaMemsetAsync(h->t2p.data, 0, bytes, h->ctx->stream));
  if (h->t1M > 0) {
    // current and previous output maps of the T1 GEMM, and T1 itself, start at zero: the
    // regions outside the current map then always hold zeros (the GEMM re-zeroes regions
    // the previous apply wrote), so the fused mix may read any input without testing it
    const size_t mb = outmap_bytes(h->t1M, h->t1N);
    h->t1map = (uint32_t*)dalloc(h, 2 * mb);
    GB_CHECK_CUDA(cudaMemsetAsync(h->t1map, 0, 2 * mb, h->ctx->stream));
    GB_REQUIRE(h->t1, "heff: T1 buffer missing");
    GB_CHECK_CUDA(cudaMemsetAsync(h->t1, 0, (size_t)h->t1M * h->t1N * sizeof(float),
                                  h->ctx->stream));
    h->t2prev = (uint32_t*)dalloc(h, (size_t)h->t2p.mrows * h->t2p.kw * 4);
    const size_t ni = h->t1roff.size();
    h->t1rc_dev = (int64_t*)dalloc(h, 2 * ni * sizeof(int64_t));
    std::vector<int64_t> rc(h->t1roff);
    rc.insert(rc.end(), h->t1coff.begin(), h->t1coff.end());
    GB_CHECK_CUDA(cudaMemcpyAsync(h->t1rc_dev, rc.data(), rc.size() * sizeof(int64_t),
                                  cudaMemcpyHostToDevice, h->ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(h->ctx->stream));
  }
  h->t2p_ready = true;
}

static void prepack(gb_heff* h, Step& s) {
  if (h->prec == GB_PREC_FP64) {
    s.hasPA = s.hasPB = false;
    return;
  }
  prepare_t2p(h);
  gb_ctx* ctx = h->ctx;
  if (s.srcA == S_CONST && !s.hasPA) {
    void* dst = dalloc(h, packed_bytes(s.M, s.K, is_cplx(h->dtype), PACK_AS_A, 1, h->prec));
    pack_operand(ctx, h->dtype, PACK_AS_A, s.opA, s.M, s.K, s.cA, s.lda, 0, 1, s.pA, dst,
                 h->prec);
    s.hasPA = true;
  }
  if (s.srcB == S_CONST && !s.hasPB) {
    void* dst = dalloc(h, packed_bytes(s.N, s.K, is_cplx(h->dtype), PACK_AS_B, 1, h->prec));
    pack_operand(ctx, h->dtype, PACK_AS_B, s.opB, s.N, s.K, s.cB, s.ldb, 0, 1, s.pB, dst,
                 h->prec);
    s.hasPB = true;
  }
}

static void ensure_prepacked(gb_heff* h);

static void free_steps(gb_heff* h) {
  for (auto& s : h->steps)
    if (!s.is_gemm) mix_free(s.mix);
  for (void* p : h->owned) cudaFreeAsync(p, h->ctx->stream);
  h->owned.clear();
  h->steps.clear();
}

static HostW hostw(const gb_tensor* W) {
  HostW w;
  w.wl = W->dims[0];
  w.d1 = W->dims[1];
  w.d2 = W->dims[2];
  w.wr = W->dims[3];
  w.cplx = is_cplx(W->dtype);
  w.v = &W->host_mpo;
  return w;
}

// ------------------------------------------------------------------ AC2
// generic: MPO_AC2_Hamiltonian of an arbitrary MPO (mpo_derivatives.jl:56-66, 144-163):
// every channel continues, no Jordan terms -- the whole operator is the x.GR -> (W1 W2) ->
// GL.(.) chain over all channels (connected ones only)
static void build_ac2(gb_heff* h, const gb_tensor* GL, const gb_tensor* W1,
                      const gb_tensor* W2, const gb_tensor* GR, bool generic = false) {
  gb_ctx* ctx = h->ctx;
  const bool cx = is_cplx(h->dtype);
  const size_t es = elem_size(h->dtype);
  HostW w1 = hostw(W1), w2 = hostw(W2);
  const int64_t Dl = GL->dims[0], wl = GL->dims[1];
  const int64_t Dr = GR->dims[0], wr = GR->dims[1];
  const int64_t d1 = w1.d1, d2 = w2.d1, wm = w1.wr;
  GB_REQUIRE(GL->dims[2] == Dl && GR->dims[2] == Dr, "AC2: bra and ket bonds must agree");
  GB_REQUIRE(w1.wl == wl && w2.wr == wr && w2.wl == wm, "AC2: MPO channel mismatch");
  GB_REQUIRE(w1.d1 == w1.d2 && w2.d1 == w2.d2, "AC2: MPO physical legs");
  const double* gl = (const double*)GL->data;
  const double* gr = (const double*)GR->data;

  // Jordan blocks (flat channel index; first = start, last = finished); for a generic MPO
  // the "continuing" block is the whole tensor (channel offset co = 0, all channels)
  const int64_t co = generic ? 0 : 1, cut = generic ? 0 : 2;
  auto A1nz = [&](int64_t c, int64_t k) {  // A1[c, :, :, k] nonzero, c < wl-2, k < wm-2
    for (int64_t s = 0; s < d1; ++s)
      for (int64_t t = 0; t < d1; ++t)
        if (w1.nz(co + c, s, t, co + k)) return true;
    return false;
  };
  auto A2nz = [&](int64_t k, int64_t m) {
    for (int64_t s = 0; s < d2; ++s)
      for (int64_t t = 0; t < d2; ++t)
        if (w2.nz(co + k, s, t, co + m)) return true;
    return false;
  };
  const int64_t nA1r = std::max<int64_t>(wl - cut, 0), nA1c = std::max<int64_t>(wm - cut, 0);
  const int64_t nA2r = nA1c, nA2c = std::max<int64_t>(wr - cut, 0);
  bool nzA1 = false, nzA2 = false, nzB1 = false, nzB2 = false, nzC1 = false, nzC2 = false,
       nzD1 = false, nzD2 = false;
  for (int64_t c = 0; c < nA1r; ++c)
    for (int64_t k = 0; k < nA1c; ++k) nzA1 |= A1nz(c, k);
  for (int64_t k = 0; k < nA2r; ++k)
    for (int64_t m = 0; m < nA2c; ++m) nzA2 |= A2nz(k, m);
  if (!generic) {
    for (int64_t s = 0; s < d1; ++s)
      for (int64_t t = 0; t < d1; ++t) {
        for (int64_t c = 0; c < nA1r; ++c) nzB1 |= w1.nz(1 + c, s, t, wm - 1);
        for (int64_t k = 0; k < nA1c; ++k) nzC1 |= w1.nz(0, s, t, 1 + k);
        nzD1 |= w1.nz(0, s, t, wm - 1);
      }
    for (int64_t s = 0; s < d2; ++s)
      for (int64_t t = 0; t < d2; ++t) {
        for (int64_t k = 0; k < nA2r; ++k) nzB2 |= w2.nz(1 + k, s, t, wr - 1);
        for (int64_t m = 0; m < nA2c; ++m) nzC2 |= w2.nz(0, s, t, 1 + m);
        nzD2 |= w2.nz(0, s, t, wr - 1);
      }
  }
  // term presence (hamiltonian_derivatives.jl:283-359); none but the chain when generic
  bool II = !generic && wr > 1, EE = !generic && wl > 1, IC = nzC2, DE = nzD1, ID = nzD2;
  bool CB = nzC1 && nzB2, CA = nzC1 && nzA2, AB = nzA1 && nzB2, BE = nzB1;
  // connected channels (:243-270)
  std::vector<int64_t> rows, mids, cols;
  if (nzA1 && nzA2) {
    std::vector<char> fed(nA1c, 0), feeds(nA1c, 0);
    for (int64_t c = 0; c < nA1r; ++c)
      for (int64_t k = 0; k < nA1c; ++k)
        if (A1nz(c, k)) fed[k] = 1;
    for (int64_t k = 0; k < nA2r; ++k)
      for (int64_t m = 0; m < nA2c; ++m)
        if (A2nz(k, m)) feeds[k] = 1;
    for (int64_t k = 0; k < nA1c; ++k)
      if (fed[k] && feeds[k]) mids.push_back(k);
    if (!mids.empty()) {
      for (int64_t c = 0; c < nA1r; ++c) {
        bool any = false;
        for (int64_t k : mids) any |= A1nz(c, k);
        if (any) rows.push_back(c);
      }
      for (int64_t m = 0; m < nA2c; ++m) {
        bool any = false;
        for (int64_t k : mids) any |= A2nz(k, m);
        if (any) cols.push_back(m);
      }
    }
  }
  bool AA = !mids.empty();

  // prepare folds (:371-468) -- decide where each cheap term goes
  enum { KEEP, INTO_CA, INTO_AB, INTO_IC, INTO_BE };
  int fCB = KEEP, fIC = KEEP, fBE = KEEP, fDE = KEEP, fID = KEEP, fII = KEEP, fEE = KEEP;
  if (CB) fCB = CA ? INTO_CA : (AB ? INTO_AB : KEEP);
  if (IC && CA) fIC = INTO_CA;
  if (BE && AB) fBE = INTO_AB;
  bool IC_live = IC && fIC == KEEP, BE_live = BE && fBE == KEEP;
  if (DE) fDE = BE_live ? INTO_BE : (AB ? INTO_AB : KEEP);
  if (ID) fID = IC_live ? INTO_IC : (CA ? INTO_CA : KEEP);
  if (II) fII = IC_live ? INTO_IC : (CA ? INTO_CA : KEEP);
  if (EE) fEE = BE_live ? INTO_BE : (AB ? INTO_AB : KEEP);

  auto C1v = [&](int64_t s, int64_t t, int64_t k) { return w1.at(0, s, t, 1 + k); };
  auto D1v = [&](int64_t s, int64_t t) { return w1.at(0, s, t, wm - 1); };
  auto B1v = [&](int64_t c, int64_t s, int64_t t) { return w1.at(1 + c, s, t, wm - 1); };
  auto A1v = [&](int64_t c, int64_t s, int64_t t, int64_t k) { return w1.at(co + c, s, t, co + k); };
  auto C2v = [&](int64_t s, int64_t t, int64_t m) { return w2.at(0, s, t, 1 + m); };
  auto D2v = [&](int64_t s, int64_t t) { return w2.at(0, s, t, wr - 1); };
  auto B2v = [&](int64_t k, int64_t s, int64_t t) { return w2.at(1 + k, s, t, wr - 1); };
  auto A2v = [&](int64_t k, int64_t s, int64_t t, int64_t m) { return w2.at(co + k, s, t, co + m); };
  auto CBv = [&](int64_t s1, int64_t s2, int64_t u1, int64_t u2) {
    Cx acc;
    for (int64_t k = 0; k < nA1c; ++k) acc = cadd(acc, cmul(C1v(s1, u1, k), B2v(k, s2, u2)));
    return acc;
  };
  auto put = [&](std::vector<double>& vals, std::vector<int64_t>& offs, int64_t off, Cx v) {
    if (v.re == 0.0 && v.im == 0.0) return;
    offs.push_back(off);
    vals.push_back(v.re);
    if (cx) vals.push_back(v.im);
  };

  std::vector<std::string> names;
  std::vector<Step> steps;
  bool y_written = false;
  auto push_gemm = [&](Step s) {
    s.accumulate = (s.dst == S_Y) ? y_written : false;
    if (s.dst == S_Y) y_written = true;
    add_gemm_flops(h, s);
    steps.push_back(s);
  };

  // in_off for GR channels and GL channels
  std::vector<int64_t> gr_in(wr), gl_in(wl);
  for (int64_t w = 0; w < wr; ++w) gr_in[w] = Dr * w;
  for (int64_t w = 0; w < wl; ++w) gl_in[w] = Dl * Dl * w;

  // ---------------- AA : continuing - continuing
  if (AA) {
    const int64_t chr = rows.size(), chc = cols.size();
    // GRc (r', j, r) and GLc (l, l', i) gathers
    void* grc = dalloc(h, (size_t)Dr * chc * Dr * es);
    void* glc = dalloc(h, (size_t)Dl * Dl * chr * es);
    {
      Coef cf(chc, wr);
      std::vector<int64_t> oo(chc);
      for (int64_t j = 0; j < chc; ++j) {
        cf.at(j, co + cols[j]) = Cx{1, 0};
        oo[j] = Dr * j;
      }
      MixDev m = mix_upload(ctx, make_plan(cf, cx, Dr, Dr, 1, Dr * wr, 1, Dr * chc, gr_in, oo));
      mix_run(ctx, m, h->dtype, gr, grc, 0.0);
      GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
      mix_free(m);
    }
    {
      Coef cf(chr, wl);
      std::vector<int64_t> oo(chr);
      for (int64_t i = 0; i < chr; ++i) {
        cf.at(i, co + rows[i]) = Cx{1, 0};
        oo[i] = Dl * Dl * i;
      }
      MixDev m = mix_upload(ctx, make_plan(cf, cx, Dl, Dl, 1, Dl, 1, Dl, gl_in, oo));
      mix_run(ctx, m, h->dtype, gl, glc, 0.0);
      GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
      mix_free(m);
    }
    // step 1: T1[(l' s1' s2'), (c' r)] = X[(l' s1' s2'), r'] . GRc[r', (c' r)]
    Step s1;
    s1.name = "AA1";
    s1.srcA = S_X;
    s1.lda = Dl * d1 * d2;
    s1.srcB = S_CONST;
    s1.cB = grc;
    s1.ldb = Dr;
    s1.dst = S_T1;
    s1.ldc = Dl * d1 * d2;
    s1.M = Dl * d1 * d2;
    s1.N = chc * Dr;
    s1.K = Dr;
    push_gemm(s1);
    h->t1_elems = std::max(h->t1_elems, s1.M * s1.N);
    // step 2: T2[l', (c s1 s2), r] = sum W12[(c s1 s2),(s1' s2' c')] T1[l', (s1' s2' c'), r]
    Coef cf(chr * d1 * d2, d1 * d2 * chc);
    for (int64_t c = 0; c < chr; ++c)
      for (int64_t sa = 0; sa < d1; ++sa)
        for (int64_t sb = 0; sb < d2; ++sb)
          for (int64_t ua = 0; ua < d1; ++ua)
            for (int64_t ub = 0; ub < d2; ++ub)
              for (int64_t j = 0; j < chc; ++j) {
                Cx acc;
                for (int64_t k : mids)
                  acc = cadd(acc, cmul(A1v(rows[c], sa, ua, k), A2v(k, sb, ub, cols[j])));
                cf.at(c + chr * (sa + d1 * sb), ua + d1 * (ub + d2 * j)) = acc;
              }
    std::vector<int64_t> io(d1 * d2 * chc), oo(chr * d1 * d2);
    for (int64_t i = 0; i < (int64_t)io.size(); ++i) io[i] = Dl * i;
    for (int64_t j = 0; j < (int64_t)oo.size(); ++j) oo[j] = Dl * j;
    record_t1_geometry(h, s1.M, s1.N, io, chc);
    Step s2;
    s2.is_gemm = false;
    s2.name = "AA2";
    s2.src = S_T1;
    s2.dst = S_T2;
    s2.mixh = make_plan(cf, cx, Dl, Dr, 1, Dl * d1 * d2 * chc, 1, Dl * chr * d1 * d2, io, oo);
    s2.mix = mix_upload(ctx, s2.mixh);
    s2.accumulate = false;
    s2.t2_producer = true;
    steps.push_back(s2);
    h->t2_elems = std::max(h->t2_elems, Dl * chr * d1 * d2 * Dr);
    // T2 as the B operand of step 3: k = l' + Dl*c, column = (s1 + d1*s2) + d1*d2*r
    h->kJ.resize(chr * d1 * d2);
    h->mJ.resize(chr * d1 * d2);
    for (int64_t c = 0; c < chr; ++c)
      for (int64_t sa = 0; sa < d1; ++sa)
        for (int64_t sb = 0; sb < d2; ++sb) {
          int64_t J = c + chr * (sa + d1 * sb);
          h->kJ[J] = Dl * c;
          h->mJ[J] = sa + d1 * sb;
        }
    h->mn = d1 * d2;
    h->t2K = Dl * chr;
    h->t2N = d1 * d2 * Dr;
    h->aa_glc = glc;
    h->aa_chr = chr;
    h->aa_grc = grc;
    h->aa_chc = chc;
    h->aa_Dl = Dl;
    h->aa_Dr = Dr;
    h->aa_np = d1 * d2;
    h->Jc.resize(chr * d1 * d2);
    h->Jp.resize(chr * d1 * d2);
    for (int64_t J = 0; J < chr * d1 * d2; ++J) {
      h->Jc[J] = J % chr;
      h->Jp[J] = J / chr;  // sa + d1 * sb
    }
    // step 3: Y[l, (s1 s2 r)] (+)= GLc[l, (l' c)] . T2[(l' c), (s1 s2 r)]
    Step s3;
    s3.name = "AA3";
    s3.srcA = S_CONST;
    s3.cA = glc;
    s3.lda = Dl;
    s3.srcB = S_T2;
    s3.ldb = Dl * chr;
    s3.dst = S_Y;
    s3.ldc = Dl;
    s3.M = Dl;
    s3.N = d1 * d2 * Dr;
    s3.K = Dl * chr;
    s3.t2_consumer = true;
    push_gemm(s3);
    names.push_back("AA");
  }

  // ---------------- CA : starting left - continuing right (3,3 tensor)
  if (CA) {
    const int64_t P = d1 * d2 * Dr;
    void* cam = dalloc(h, (size_t)P * P * es);
    Coef cf(d1 * d2 * d1 * d2, wr);  // J = (s1', s2', s1, s2)
    auto J = [&](int64_t u1, int64_t u2, int64_t s1, int64_t s2) {
      return u1 + d1 * (u2 + d2 * (s1 + d1 * s2));
    };
    std::vector<double> dv;
    std::vector<int64_t> doff;
    std::vector<int64_t> oo(cf.nJ);
    for (int64_t s1 = 0; s1 < d1; ++s1)
      for (int64_t s2 = 0; s2 < d2; ++s2)
        for (int64_t u1 = 0; u1 < d1; ++u1)
          for (int64_t u2 = 0; u2 < d2; ++u2) {
            int64_t j = J(u1, u2, s1, s2);
            oo[j] = u1 + d1 * u2 + d1 * d2 * Dr * s1 + d1 * d1 * d2 * Dr * s2;
            for (int64_t m = 0; m < nA2c; ++m) {
              Cx acc;
              for (int64_t k = 0; k < nA1c; ++k)
                acc = cadd(acc, cmul(C1v(s1, u1, k), A2v(k, s2, u2, m)));
              if (fIC == INTO_CA && s1 == u1) acc = cadd(acc, C2v(s2, u2, m));
              cf.at(j, 1 + m) = acc;
            }
            if (fII == INTO_CA && s1 == u1 && s2 == u2) cf.at(j, 0) = cadd(cf.at(j, 0), Cx{1, 0});
            Cx dg;
            if (fCB == INTO_CA) dg = cadd(dg, CBv(s1, s2, u1, u2));
            if (fID == INTO_CA && s1 == u1) dg = cadd(dg, D2v(s2, u2));
            put(dv, doff, oo[j], dg);
          }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dr, Dr, 1, Dr * wr, d1 * d2,
                                         d1 * d1 * d2 * d2 * Dr, gr_in, oo));
    mix_run(ctx, m, h->dtype, gr, cam, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, cam, doff, dv, Dr, d1 * d2 + d1 * d1 * d2 * d2 * Dr);
    Step s;
    s.name = "CA";
    s.srcA = S_X;
    s.lda = Dl;
    s.srcB = S_CONST;
    s.cB = cam;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = Dl;
    s.M = Dl;
    s.N = P;
    s.K = P;
    push_gemm(s);
    names.push_back("CA");
  }

  // ---------------- AB : continuing left - ending right (3,3 tensor)
  if (AB) {
    const int64_t P = Dl * d1 * d2;
    void* abm = dalloc(h, (size_t)P * P * es);
    Coef cf(d1 * d2 * d1 * d2, wl);  // J = (s1, s2, s1', s2')
    std::vector<double> dv;
    std::vector<int64_t> doff;
    std::vector<int64_t> oo(cf.nJ);
    for (int64_t s1 = 0; s1 < d1; ++s1)
      for (int64_t s2 = 0; s2 < d2; ++s2)
        for (int64_t u1 = 0; u1 < d1; ++u1)
          for (int64_t u2 = 0; u2 < d2; ++u2) {
            int64_t j = s1 + d1 * (s2 + d2 * (u1 + d1 * u2));
            oo[j] = Dl * s1 + Dl * d1 * s2 + Dl * Dl * d1 * d2 * u1 + Dl * Dl * d1 * d1 * d2 * u2;
            for (int64_t c = 0; c < nA1r; ++c) {
              Cx acc;
              for (int64_t k = 0; k < nA1c; ++k)
                acc = cadd(acc, cmul(A1v(c, s1, u1, k), B2v(k, s2, u2)));
              if (fBE == INTO_AB && s2 == u2) acc = cadd(acc, B1v(c, s1, u1));
              cf.at(j, 1 + c) = acc;
            }
            if (fEE == INTO_AB && s1 == u1 && s2 == u2)
              cf.at(j, wl - 1) = cadd(cf.at(j, wl - 1), Cx{1, 0});
            Cx dg;
            if (fCB == INTO_AB) dg = cadd(dg, CBv(s1, s2, u1, u2));
            if (fDE == INTO_AB && s2 == u2) dg = cadd(dg, D1v(s1, u1));
            put(dv, doff, oo[j], dg);
          }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dl, Dl, 1, Dl, 1, Dl * d1 * d2, gl_in, oo));
    mix_run(ctx, m, h->dtype, gl, abm, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, abm, doff, dv, Dl, 1 + Dl * d1 * d2);
    Step s;
    s.name = "AB";
    s.srcA = S_CONST;
    s.cA = abm;
    s.lda = P;
    s.srcB = S_X;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = P;
    s.M = P;
    s.N = Dr;
    s.K = P;
    push_gemm(s);
    names.push_back("AB");
  }

  // ---------------- IC : starting right (2,2 tensor)
  if (IC && fIC == KEEP) {
    const int64_t P = d2 * Dr;
    void* icm = dalloc(h, (size_t)P * P * es);
    Coef cf(d2 * d2, wr);  // J = (s2', s2)
    std::vector<double> dv;
    std::vector<int64_t> doff;
    std::vector<int64_t> oo(cf.nJ);
    for (int64_t s2 = 0; s2 < d2; ++s2)
      for (int64_t u2 = 0; u2 < d2; ++u2) {
        int64_t j = u2 + d2 * s2;
        oo[j] = u2 + d2 * Dr * s2;
        for (int64_t m = 0; m < nA2c; ++m) cf.at(j, 1 + m) = C2v(s2, u2, m);
        if (fII == INTO_IC && s2 == u2) cf.at(j, 0) = cadd(cf.at(j, 0), Cx{1, 0});
        Cx dg;
        if (fID == INTO_IC) dg = D2v(s2, u2);
        put(dv, doff, oo[j], dg);
      }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dr, Dr, 1, Dr * wr, d2, d2 * d2 * Dr, gr_in, oo));
    mix_run(ctx, m, h->dtype, gr, icm, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, icm, doff, dv, Dr, d2 + d2 * d2 * Dr);
    Step s;
    s.name = "IC";
    s.srcA = S_X;
    s.lda = Dl * d1;
    s.srcB = S_CONST;
    s.cB = icm;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = Dl * d1;
    s.M = Dl * d1;
    s.N = P;
    s.K = P;
    push_gemm(s);
    names.push_back("IC");
  }

  // ---------------- BE : ending left (2,2 tensor)
  if (BE && fBE == KEEP) {
    const int64_t P = Dl * d1;
    void* bem = dalloc(h, (size_t)P * P * es);
    Coef cf(d1 * d1, wl);  // J = (s1, s1')
    std::vector<double> dv;
    std::vector<int64_t> doff;
    std::vector<int64_t> oo(cf.nJ);
    for (int64_t s1 = 0; s1 < d1; ++s1)
      for (int64_t u1 = 0; u1 < d1; ++u1) {
        int64_t j = s1 + d1 * u1;
        oo[j] = Dl * s1 + Dl * Dl * d1 * u1;
        for (int64_t c = 0; c < nA1r; ++c) cf.at(j, 1 + c) = B1v(c, s1, u1);
        if (fEE == INTO_BE && s1 == u1) cf.at(j, wl - 1) = cadd(cf.at(j, wl - 1), Cx{1, 0});
        Cx dg;
        if (fDE == INTO_BE) dg = D1v(s1, u1);
        put(dv, doff, oo[j], dg);
      }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dl, Dl, 1, Dl, 1, Dl * d1, gl_in, oo));
    mix_run(ctx, m, h->dtype, gl, bem, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, bem, doff, dv, Dl, 1 + Dl * d1);
    Step s;
    s.name = "BE";
    s.srcA = S_CONST;
    s.cA = bem;
    s.lda = P;
    s.srcB = S_X;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = P;
    s.M = P;
    s.N = d2 * Dr;
    s.K = P;
    push_gemm(s);
    names.push_back("BE");
  }

  // ---------------- leftover cheap terms
  if (II && fII == KEEP) {  // Y[(l s1 s2), r] += X[(l s1 s2), r'] GR[r', 0, r]
    Step s;
    s.name = "II";
    s.srcA = S_X;
    s.lda = Dl * d1 * d2;
    s.srcB = S_CONST;
    s.cB = gr;
    s.ldb = Dr * wr;
    s.dst = S_Y;
    s.ldc = Dl * d1 * d2;
    s.M = Dl * d1 * d2;
    s.N = Dr;
    s.K = Dr;
    push_gemm(s);
    names.push_back("II");
  }
  if (EE && fEE == KEEP) {  // Y[l, (s1 s2 r)] += GL[:, :, end] X[l', (s1 s2 r)]
    Step s;
    s.name = "EE";
    s.srcA = S_CONST;
    s.cA = (const char*)gl + (size_t)Dl * Dl * (wl - 1) * es;
    s.lda = Dl;
    s.srcB = S_X;
    s.ldb = Dl;
    s.dst = S_Y;
    s.ldc = Dl;
    s.M = Dl;
    s.N = d1 * d2 * Dr;
    s.K = Dl;
    push_gemm(s);
    names.push_back("EE");
  }
  auto push_mix = [&](const char* nm, const Coef& cf, int64_t A, int64_t N, int64_t xn,
                      const std::vector<int64_t>& io, const std::vector<int64_t>& oo) {
    Step s;
    s.is_gemm = false;
    s.name = nm;
    s.src = S_X;
    s.dst = S_Y;
    s.mix = mix_upload(ctx, make_plan(cf, cx, A, N, 1, xn, 1, xn, io, oo));
    s.accumulate = true;
    if (!y_written) h->y_zero_first = true;
    steps.push_back(s);
    names.push_back(nm);
  };
  if (ID && fID == KEEP) {  // mix on s2: a = (l s1), n = r
    Coef cf(d2, d2);
    std::vector<int64_t> io(d2), oo(d2);
    for (int64_t s = 0; s < d2; ++s) {
      io[s] = oo[s] = Dl * d1 * s;
      for (int64_t u = 0; u < d2; ++u) cf.at(s, u) = D2v(s, u);
    }
    push_mix("ID", cf, Dl * d1, Dr, Dl * d1 * d2, io, oo);
  }
  if (DE && fDE == KEEP) {  // mix on s1: a = l, n = (s2 r)
    Coef cf(d1, d1);
    std::vector<int64_t> io(d1), oo(d1);
    for (int64_t s = 0; s < d1; ++s) {
      io[s] = oo[s] = Dl * s;
      for (int64_t u = 0; u < d1; ++u) cf.at(s, u) = D1v(s, u);
    }
    push_mix("DE", cf, Dl, d2 * Dr, Dl * d1, io, oo);
  }
  if (CB && fCB == KEEP) {  // mix on (s1, s2): a = l, n = r
    Coef cf(d1 * d2, d1 * d2);
    std::vector<int64_t> io(d1 * d2), oo(d1 * d2);
    for (int64_t s1 = 0; s1 < d1; ++s1)
      for (int64_t s2 = 0; s2 < d2; ++s2) {
        int64_t j = s1 + d1 * s2;
        io[j] = oo[j] = Dl * s1 + Dl * d1 * s2;
        for (int64_t u1 = 0; u1 < d1; ++u1)
          for (int64_t u2 = 0; u2 < d2; ++u2) cf.at(j, u1 + d1 * u2) = CBv(s1, s2, u1, u2);
      }
    push_mix("CB", cf, Dl, Dr, Dl * d1 * d2, io, oo);
  }
  if (!y_written && steps.empty()) h->y_zero_first = true;
  // mixes before any GEMM wrote y need y zeroed; GEMMs after a mix accumulate
  h->steps = std::move(steps);
  // report the terms in the reference's field order (hamiltonian_derivatives.jl:168-178)
  static const char* order[] = {"II", "IC", "ID", "CB", "CA", "AB", "AA", "BE", "DE", "EE"};
  std::vector<std::string> sorted;
  for (const char* o : order)
    if (std::find(names.begin(), names.end(), o) != names.end()) sorted.push_back(o);
  names = sorted;
  std::ostringstream os;
  for (size_t i = 0; i < names.size(); ++i) os << (i ? "," : "") << names[i];
  h->terms = os.str();
  h->xndim = 4;
  h->xdims[0] = Dl;
  h->xdims[1] = d1;
  h->xdims[2] = Dr;
  h->xdims[3] = d2;
  h->xnumel = Dl * d1 * d2 * Dr;
}

// ------------------------------------------------------------------ AC
// generic: MPO_AC_Hamiltonian of an arbitrary MPO (mpo_derivatives.jl:46-55, 127-142): no
// Jordan terms, the whole operator is the x.GR -> W -> GL.(.) chain over all channels
static void build_ac(gb_heff* h, const gb_tensor* GL, const gb_tensor* W, const gb_tensor* GR,
                     bool generic = false) {
  gb_ctx* ctx = h->ctx;
  const bool cx = is_cplx(h->dtype);
  const size_t es = elem_size(h->dtype);
  HostW w = hostw(W);
  const int64_t Dl = GL->dims[0], wl = GL->dims[1];
  const int64_t Dr = GR->dims[0], wr = GR->dims[1];
  const int64_t d = w.d1;
  GB_REQUIRE(GL->dims[2] == Dl && GR->dims[2] == Dr, "AC: bra and ket bonds must agree");
  GB_REQUIRE(w.wl == wl && w.wr == wr && w.d1 == w.d2, "AC: MPO shape mismatch");
  const double* gl = (const double*)GL->data;
  const double* gr = (const double*)GR->data;
  const int64_t co = generic ? 0 : 1, cut = generic ? 0 : 2;
  const int64_t nr = std::max<int64_t>(wl - cut, 0), nc = std::max<int64_t>(wr - cut, 0);
  auto Av = [&](int64_t c, int64_t s, int64_t t, int64_t k) { return w.at(co + c, s, t, co + k); };
  auto Bv = [&](int64_t c, int64_t s, int64_t t) { return w.at(1 + c, s, t, wr - 1); };
  auto Cv = [&](int64_t s, int64_t t, int64_t k) { return w.at(0, s, t, 1 + k); };
  auto Dv = [&](int64_t s, int64_t t) { return w.at(0, s, t, wr - 1); };
  bool nzA = false, nzB = false, nzC = false, nzD = false;
  std::vector<char> rowA(nr, 0), colA(nc, 0);
  for (int64_t s = 0; s < d; ++s)
    for (int64_t t = 0; t < d; ++t) {
      for (int64_t c = 0; c < nr; ++c)
        for (int64_t k = 0; k < nc; ++k)
          if (w.nz(co + c, s, t, co + k)) {
            nzA = true;
            rowA[c] = 1;
            colA[k] = 1;
          }
      if (generic) continue;
      for (int64_t c = 0; c < nr; ++c) nzB |= w.nz(1 + c, s, t, wr - 1);
      for (int64_t k = 0; k < nc; ++k) nzC |= w.nz(0, s, t, 1 + k);
      nzD |= w.nz(0, s, t, wr - 1);
    }
  bool D = nzD, I = !generic && wr > 1, E = !generic && wl > 1, C = nzC, B = nzB, A = nzA;
  enum { KEEP, INTO_C, INTO_B };
  int fD = KEEP, fI = KEEP, fE = KEEP;
  if (D) fD = C ? INTO_C : (B ? INTO_B : KEEP);
  if (I && C) fI = INTO_C;
  if (E && B) fE = INTO_B;
  auto put = [&](std::vector<double>& vals, std::vector<int64_t>& offs, int64_t off, Cx v) {
    if (v.re == 0.0 && v.im == 0.0) return;
    offs.push_back(off);
    vals.push_back(v.re);
    if (cx) vals.push_back(v.im);
  };
  std::vector<int64_t> gr_in(wr), gl_in(wl);
  for (int64_t q = 0; q < wr; ++q) gr_in[q] = Dr * q;
  for (int64_t q = 0; q < wl; ++q) gl_in[q] = Dl * Dl * q;
  std::vector<std::string> names;
  std::vector<Step> steps;
  bool y_written = false;
  auto push_gemm = [&](Step s) {
    s.accumulate = (s.dst == S_Y) ? y_written : false;
    if (s.dst == S_Y) y_written = true;
    add_gemm_flops(h, s);
    steps.push_back(s);
  };
  if (A) {
    std::vector<int64_t> rows, cols;
    for (int64_t c = 0; c < nr; ++c)
      if (rowA[c]) rows.push_back(c);
    for (int64_t k = 0; k < nc; ++k)
      if (colA[k]) cols.push_back(k);
    const int64_t chr = rows.size(), chc = cols.size();
    void* grc = dalloc(h, (size_t)Dr * chc * Dr * es);
    void* glc = dalloc(h, (size_t)Dl * Dl * chr * es);
    {
      Coef cf(chc, wr);
      std::vector<int64_t> oo(chc);
      for (int64_t j = 0; j < chc; ++j) {
        cf.at(j, co + cols[j]) = Cx{1, 0};
        oo[j] = Dr * j;
      }
      MixDev m = mix_upload(ctx, make_plan(cf, cx, Dr, Dr, 1, Dr * wr, 1, Dr * chc, gr_in, oo));
      mix_run(ctx, m, h->dtype, gr, grc, 0.0);
      GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
      mix_free(m);
    }
    {
      Coef cf(chr, wl);
      std::vector<int64_t> oo(chr);
      for (int64_t i = 0; i < chr; ++i) {
        cf.at(i, co + rows[i]) = Cx{1, 0};
        oo[i] = Dl * Dl * i;
      }
      MixDev m = mix_upload(ctx, make_plan(cf, cx, Dl, Dl, 1, Dl, 1, Dl, gl_in, oo));
      mix_run(ctx, m, h->dtype, gl, glc, 0.0);
      GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
      mix_free(m);
    }
    Step s1;
    s1.name = "A1";
    s1.srcA = S_X;
    s1.lda = Dl * d;
    s1.srcB = S_CONST;
    s1.cB = grc;
    s1.ldb = Dr;
    s1.dst = S_T1;
    s1.ldc = Dl * d;
    s1.M = Dl * d;
    s1.N = chc * Dr;
    s1.K = Dr;
    push_gemm(s1);
    h->t1_elems = std::max(h->t1_elems, s1.M * s1.N);
    Coef cf(chr * d, d * chc);
    for (int64_t c = 0; c < chr; ++c)
      for (int64_t s = 0; s < d; ++s)
        for (int64_t u = 0; u < d; ++u)
          for (int64_t j = 0; j < chc; ++j) cf.at(c + chr * s, u + d * j) = Av(rows[c], s, u, cols[j]);
    std::vector<int64_t> io(d * chc), oo(chr * d);
    for (int64_t i = 0; i < (int64_t)io.size(); ++i) io[i] = Dl * i;
    for (int64_t j = 0; j < (int64_t)oo.size(); ++j) oo[j] = Dl * j;
    record_t1_geometry(h, s1.M, s1.N, io, chc);
    Step s2;
    s2.is_gemm = false;
    s2.name = "A2";
    s2.src = S_T1;
    s2.dst = S_T2;
    s2.mixh = make_plan(cf, cx, Dl, Dr, 1, Dl * d * chc, 1, Dl * chr * d, io, oo);
    s2.mix = mix_upload(ctx, s2.mixh);
    s2.accumulate = false;
    s2.t2_producer = true;
    steps.push_back(s2);
    h->t2_elems = std::max(h->t2_elems, Dl * chr * d * Dr);
    h->kJ.resize(chr * d);
    h->mJ.resize(chr * d);
    for (int64_t c = 0; c < chr; ++c)
      for (int64_t sa = 0; sa < d; ++sa) {
        h->kJ[c + chr * sa] = Dl * c;
        h->mJ[c + chr * sa] = sa;
      }
    h->mn = d;
    h->t2K = Dl * chr;
    h->t2N = d * Dr;
    h->aa_glc = glc;
    h->aa_chr = chr;
    h->aa_grc = grc;
    h->aa_chc = chc;
    h->aa_Dl = Dl;
    h->aa_Dr = Dr;
    h->aa_np = d;
    h->Jc.resize(chr * d);
    h->Jp.resize(chr * d);
    for (int64_t J = 0; J < chr * d; ++J) {
      h->Jc[J] = J % chr;
      h->Jp[J] = J / chr;
    }
    Step s3;
    s3.name = "A3";
    s3.srcA = S_CONST;
    s3.cA = glc;
    s3.lda = Dl;
    s3.srcB = S_T2;
    s3.ldb = Dl * chr;
    s3.dst = S_Y;
    s3.ldc = Dl;
    s3.M = Dl;
    s3.N = d * Dr;
    s3.K = Dl * chr;
    s3.t2_consumer = true;
    push_gemm(s3);
    names.push_back("A");
  }
  if (C) {  // Cm (s', r', s, r)
    const int64_t P = d * Dr;
    void* cm = dalloc(h, (size_t)P * P * es);
    Coef cf(d * d, wr);
    std::vector<double> dv;
    std::vector<int64_t> doff, oo(d * d);
    for (int64_t s = 0; s < d; ++s)
      for (int64_t u = 0; u < d; ++u) {
        int64_t j = u + d * s;
        oo[j] = u + d * Dr * s;
        for (int64_t k = 0; k < nc; ++k) cf.at(j, 1 + k) = Cv(s, u, k);
        if (fI == INTO_C && s == u) cf.at(j, 0) = cadd(cf.at(j, 0), Cx{1, 0});
        Cx dg;
        if (fD == INTO_C) dg = Dv(s, u);
        put(dv, doff, oo[j], dg);
      }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dr, Dr, 1, Dr * wr, d, d * d * Dr, gr_in, oo));
    mix_run(ctx, m, h->dtype, gr, cm, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, cm, doff, dv, Dr, d + d * d * Dr);
    Step s;
    s.name = "C";
    s.srcA = S_X;
    s.lda = Dl;
    s.srcB = S_CONST;
    s.cB = cm;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = Dl;
    s.M = Dl;
    s.N = P;
    s.K = P;
    push_gemm(s);
    names.push_back("C");
  }
  if (B) {  // Bm (l, s, l', s')
    const int64_t P = Dl * d;
    void* bm = dalloc(h, (size_t)P * P * es);
    Coef cf(d * d, wl);
    std::vector<double> dv;
    std::vector<int64_t> doff, oo(d * d);
    for (int64_t s = 0; s < d; ++s)
      for (int64_t u = 0; u < d; ++u) {
        int64_t j = s + d * u;
        oo[j] = Dl * s + Dl * Dl * d * u;
        for (int64_t c = 0; c < nr; ++c) cf.at(j, 1 + c) = Bv(c, s, u);
        if (fE == INTO_B && s == u) cf.at(j, wl - 1) = cadd(cf.at(j, wl - 1), Cx{1, 0});
        Cx dg;
        if (fD == INTO_B) dg = Dv(s, u);
        put(dv, doff, oo[j], dg);
      }
    MixDev m = mix_upload(ctx, make_plan(cf, cx, Dl, Dl, 1, Dl, 1, Dl * d, gl_in, oo));
    mix_run(ctx, m, h->dtype, gl, bm, 0.0);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    mix_free(m);
    add_diag(ctx, h->dtype, bm, doff, dv, Dl, 1 + Dl * d);
    Step s;
    s.name = "B";
    s.srcA = S_CONST;
    s.cA = bm;
    s.lda = P;
    s.srcB = S_X;
    s.ldb = P;
    s.dst = S_Y;
    s.ldc = P;
    s.M = P;
    s.N = Dr;
    s.K = P;
    push_gemm(s);
    names.push_back("B");
  }
  if (I && fI == KEEP) {
    Step s;
    s.name = "I";
    s.srcA = S_X;
    s.lda = Dl * d;
    s.srcB = S_CONST;
    s.cB = gr;
    s.ldb = Dr * wr;
    s.dst = S_Y;
    s.ldc = Dl * d;
    s.M = Dl * d;
    s.N = Dr;
    s.K = Dr;
    push_gemm(s);
    names.push_back("I");
  }
  if (E && fE == KEEP) {
    Step s;
    s.name = "E";
    s.srcA = S_CONST;
    s.cA = (const char*)gl + (size_t)Dl * Dl * (wl - 1) * es;
    s.lda = Dl;
    s.srcB = S_X;
    s.ldb = Dl;
    s.dst = S_Y;
    s.ldc = Dl;
    s.M = Dl;
    s.N = d * Dr;
    s.K = Dl;
    push_gemm(s);
    names.push_back("E");
  }
  if (D && fD == KEEP) {
    Coef cf(d, d);
    std::vector<int64_t> io(d), oo(d);
    for (int64_t s = 0; s < d; ++s) {
      io[s] = oo[s] = Dl * s;
      for (int64_t u = 0; u < d; ++u) cf.at(s, u) = Dv(s, u);
    }
    Step s;
    s.is_gemm = false;
    s.name = "D";
    s.src = S_X;
    s.dst = S_Y;
    s.mix = mix_upload(ctx, make_plan(cf, cx, Dl, Dr, 1, Dl * d, 1, Dl * d, io, oo));
    s.accumulate = true;
    if (!y_written) h->y_zero_first = true;
    steps.push_back(s);
    names.push_back("D");
  }
  if (steps.empty()) h->y_zero_first = true;
  h->steps = std::move(steps);
  // report the terms in the reference's field order (hamiltonian_derivatives.jl:15-21)
  static const char* order[] = {"D", "I", "E", "C", "B", "A"};
  std::vector<std::string> sorted;
  for (const char* o : order)
    if (std::find(names.begin(), names.end(), o) != names.end()) sorted.push_back(o);
  names = sorted;
  std::ostringstream os;
  for (size_t i = 0; i < names.size(); ++i) os << (i ? "," : "") << names[i];
  h->terms = os.str();
  h->xndim = 3;
  h->xdims[0] = Dl;
  h->xdims[1] = d;
  h->xdims[2] = Dr;
  h->xnumel = Dl * d * Dr;
}

// ------------------------------------------------------------------ C
static void build_c(gb_heff* h, const gb_tensor* GL, const gb_tensor* GR) {
  const int64_t Dl = GL->dims[0], w = GL->dims[1];
  const int64_t Dr = GR->dims[0];
  GB_REQUIRE(GR->dims[1] == w, "C: GL and GR channel mismatch");
  GB_REQUIRE(GL->dims[2] == Dl && GR->dims[2] == Dr, "C: bra and ket bonds must agree");
  bool y_written = false;
  auto push_gemm = [&](Step s) {
    s.accumulate = (s.dst == S_Y) ? y_written : false;
    if (s.dst == S_Y) y_written = true;
    add_gemm_flops(h, s);
    h->steps.push_back(s);
  };
  // T[l', (w r)] = X[l', r'] GR[r', (w r)]
  Step s1;
  s1.name = "C1";
  s1.srcA = S_X;
  s1.lda = Dl;
  s1.srcB = S_CONST;
  s1.cB = GR->data;
  s1.ldb = Dr;
  s1.dst = S_T1;
  s1.ldc = Dl;
  s1.M = Dl;
  s1.N = w * Dr;
  s1.K = Dr;
  push_gemm(s1);
  h->t1_elems = Dl * w * Dr;
  // Y[l, r] = GL[l, (l' w)] T[(l' w), r]
  Step s2;
  s2.name = "C2";
  s2.srcA = S_CONST;
  s2.cA = GL->data;
  s2.lda = Dl;
  s2.srcB = S_T1;
  s2.ldb = Dl * w;
  s2.dst = S_Y;
  s2.ldc = Dl;
  s2.M = Dl;
  s2.N = Dr;
  s2.K = Dl * w;
  push_gemm(s2);
  h->terms = "GL.x.GR";
  h->xndim = 2;
  h->xdims[0] = Dl;
  h->xdims[1] = Dr;
  h->xnumel = Dl * Dr;
}

// ------------------------------------------------------------------ public helpers
gb_heff* heff_build(gb_ctx* ctx, int kind, const gb_tensor* GL, const gb_tensor* W1,
                    const gb_tensor* W2, const gb_tensor* GR, int prec) {
  GB_REQUIRE(GL && GR, "heff: GL and GR are required");
  GB_REQUIRE(GL->kind == GB_KIND_GL && GR->kind == GB_KIND_GR, "heff: env kinds");
  GB_REQUIRE(GL->dtype == GR->dtype, "heff: GL/GR dtype mismatch");
  GB_REQUIRE(prec == GB_PREC_FP64 || prec == GB_PREC_BF16X3 || prec == GB_PREC_TF32X3,
             "heff: precision");
  for (const gb_tensor* W : {W1, W2}) {
    if (!W) continue;
    GB_REQUIRE(W->kind == GB_KIND_MPO, "heff: W must be an MPO tensor");
    GB_REQUIRE(!(is_cplx(W->dtype) && !is_cplx(GL->dtype)),
               "heff: complex MPO needs complex environments");
  }
  gb_heff* h = new gb_heff();
  h->ctx = ctx;
  h->kind = kind;
  h->dtype = GL->dtype;
  h->prec = prec;
  h->sched = ctx->gemm_schedule;
  // the generic-MPO kinds are built and applied as the Jordan kinds with one term
  const bool generic = kind == GB_HEFF_AC_MPO || kind == GB_HEFF_AC2_MPO;
  if (kind == GB_HEFF_AC_MPO) h->kind = kind = GB_HEFF_AC;
  if (kind == GB_HEFF_AC2_MPO) h->kind = kind = GB_HEFF_AC2;
  try {
    if (kind == GB_HEFF_AC2) {
      GB_REQUIRE(W1 && W2, "AC2 needs W1 and W2");
      build_ac2(h, GL, W1, W2, GR, generic);
    } else if (kind == GB_HEFF_AC) {
      GB_REQUIRE(W1 && !W2, "AC needs exactly W1");
      build_ac(h, GL, W1, GR, generic);
    } else if (kind == GB_HEFF_C) {
      GB_REQUIRE(!W1 && !W2, "C takes no MPO tensor");
      build_c(h, GL, GR);
    } else {
      throw Error(GB_ERR_ARG, "heff: unknown kind");
    }
    size_t es = elem_size(h->dtype);
    if (h->t1_elems) h->t1 = dalloc(h, (size_t)h->t1_elems * es);
    // the FP64 T2 buffer is only needed when T2 is not written packed (split precision)
    if (h->t2_elems && (h->prec == GB_PREC_FP64 || h->kJ.empty()))
      h->t2 = dalloc(h, (size_t)h->t2_elems * es);
    // with the grouped schedule a real split-precision operator packs its constants when
    // its sectors arrive (gb_heff_set_sectors); the dense-embedding packing is then only
    // made if the operator is applied without sectors
    const bool deferred = h->sched == GB_SCHED_GROUPED && h->prec != GB_PREC_FP64 &&
                          !is_cplx(h->dtype) && h->kind != GB_HEFF_C;
    if (!deferred) ensure_prepacked(h);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    free_steps(h);
    delete h;
    throw;
  }
  return h;
}

void heff_free(gb_heff* h) {
  if (!h) return;
  free_steps(h);
  delete h;
}

int heff_precision(const gb_heff* h) { return h->prec; }

// dq[c] = q_l(l) - q_l(l') over the nonzero entries of GL's continuing channel c (one
// value per channel when GL conserves charge; INT_MIN: the channel is zero)
__global__ void channel_charge_kernel(const double* __restrict__ glc, int64_t Dl, int64_t chr,
                                      int cplx, const int* __restrict__ ql, int* dq, int* bad) {
  const int64_t n = Dl * Dl * chr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const bool nz = cplx ? (glc[2 * i] != 0.0 || glc[2 * i + 1] != 0.0) : glc[i] != 0.0;
    if (!nz) continue;
    const int64_t l = i % Dl, lp = (i / Dl) % Dl, c = i / (Dl * Dl);
    const int v = ql[l] - ql[lp];
    // a plain read settles almost every entry once the channel's value is known; only the
    // first entries of a channel race on the compare-and-swap
    int cur = *(volatile int*)&dq[c];
    if (cur == INT_MIN) {
      cur = atomicCAS(&dq[c], INT_MIN, v);
      if (cur == INT_MIN) cur = v;
    }
    if (cur != v) atomicExch(bad, 1);
  }
}

void heff_apply_raw(gb_heff* h, const void* x, void* y);

template <typename T>
__global__ void runs_copy_kernel(const int64_t* __restrict__ runs, int64_t nruns,
                                 const T* __restrict__ src, T* __restrict__ dst, int scatter) {
  for (int64_t c = blockIdx.x; c < nruns; c += gridDim.x) {
    const int64_t co = runs[3 * c], dof = runs[3 * c + 1], len = runs[3 * c + 2];
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
      if (scatter) dst[dof + i] = src[co + i];
      else dst[co + i] = src[dof + i];
    }
  }
}

// compact <-> dense copies of the allowed entries (scatter = 1: compact -> dense)
static void runs_copy(gb_heff* h, const void* src, void* dst, int scatter) {
  gb_ctx* ctx = h->ctx;
  const unsigned grid = (unsigned)std::min<int64_t>(h->nruns, 152 * 8);
  if (grid == 0) return;
  if (is_cplx(h->dtype))
    runs_copy_kernel<double2><<<grid, 256, 0, ctx->stream>>>(h->runs, h->nruns,
                                                             (const double2*)src, (double2*)dst,
                                                             scatter);
  else
    runs_copy_kernel<double><<<grid, 256, 0, ctx->stream>>>(h->runs, h->nruns,
                                                            (const double*)src, (double*)dst,
                                                            scatter);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

bool heff_compact(gb_heff* h, HeffCompact* c) {
  if (!h->runs) return false;
  const size_t es = elem_size(h->dtype);
  if (!h->xfull) {
    h->xfull = dalloc(h, (size_t)h->xnumel * es);
    GB_CHECK_CUDA(cudaMemsetAsync(h->xfull, 0, (size_t)h->xnumel * es, h->ctx->stream));
    h->yfull = dalloc(h, (size_t)h->xnumel * es);
    h->xcomp = dalloc(h, (size_t)std::max<int64_t>(h->ncompact, 1) * es);
  }
  c->n = h->ncompact;
  c->xcomp = h->xcomp;
  return true;
}

void heff_gather(gb_heff* h, const void* dense, void* compact) { runs_copy(h, dense, compact, 0); }

void heff_scatter(gb_heff* h, const void* compact, void* dense) {
  fill_zero(h->ctx, dense, (size_t)h->xnumel * elem_size(h->dtype));
  runs_copy(h, compact, dense, 1);
}

// y = H x on compact vectors: scatter into the zero-padded staging vector, apply, gather
void heff_apply_compact(gb_heff* h, const void* x, void* y) {
  runs_copy(h, x, h->xfull, 1);
  heff_apply_raw(h, h->xfull, h->yfull);
  runs_copy(h, h->yfull, y, 0);
}

static void build_staged_mix(gb_heff* h, int64_t Dr);
static void grouped_prepare(gb_heff* h);

void heff_set_sectors(gb_heff* h, const int32_t* ql, const int32_t* qp1, const int32_t* qp2,
                      const int32_t* qr) {
  gb_ctx* ctx = h->ctx;
  const int64_t Dl = h->xdims[0], Dr = h->xdims[2];  // x: (l, s1, r, s2) or (l, s, r)
  for (int64_t i = 1; i < Dl; ++i)
    GB_REQUIRE(ql[i - 1] <= ql[i], "set_sectors: left charges must be sorted ascending");
  {
    const bool two = h->kind == GB_HEFF_AC2;
    h->q_l.assign(ql, ql + Dl);
    h->q_r.assign(qr, qr + Dr);
    h->q_p1.assign(qp1, qp1 + h->xdims[1]);
    if (two) {
      GB_REQUIRE(qp2, "set_sectors: two physical legs expected");
      h->q_p2.assign(qp2, qp2 + h->xdims[3]);
    } else {
      h->q_p2.clear();
    }
    h->dq_l.clear();
    h->arange_h.clear();
  }
  // sector table of the (sorted) left charges, indexed by charge - ql[0]
  const int64_t qmin = ql[0], qspan = (int64_t)ql[Dl - 1] - qmin + 1;
  std::vector<int2> sec((size_t)qspan, int2{0, 0});
  for (int64_t i = 0; i < Dl; ++i) {
    int2& r = sec[(size_t)(ql[i] - qmin)];
    if (r.y == 0) r.x = (int)i;
    r.y = (int)i + 1;
  }
  auto sector = [&](int64_t q) {
    const int64_t t = q - qmin;
    return (t >= 0 && t < qspan) ? sec[(size_t)t] : int2{0, 0};
  };
  // runs of x: device layout (l, s1, s2, r) or (l, s, r), l fastest (a later call with
  // other charges replaces them; the staging vector is then cleared again)
  {
    const bool two = h->kind == GB_HEFF_AC2;
    const int64_t d1 = h->xdims[1], d2 = two ? h->xdims[3] : 1;
    std::vector<int64_t> runs;
    int64_t off = 0;
    for (int64_t r = 0; r < Dr; ++r)
      for (int64_t s2 = 0; s2 < d2; ++s2)
        for (int64_t s1 = 0; s1 < d1; ++s1) {
          const int64_t col = s1 + d1 * (s2 + d2 * r);
          const int2 lr = sector((int64_t)qr[r] - qp1[s1] - (two ? qp2[s2] : 0));
          if (lr.y <= lr.x) continue;
          runs.push_back(off);
          runs.push_back(col * Dl + lr.x);
          runs.push_back(lr.y - lr.x);
          off += lr.y - lr.x;
        }
    GB_REQUIRE(off > 0, "set_sectors: no allowed entry (charges inconsistent with the vector)");
    h->nruns = (int64_t)runs.size() / 3;
    h->ncompact = off;
    h->runs = (int64_t*)dalloc(h, runs.size() * sizeof(int64_t));
    GB_CHECK_CUDA(cudaMemcpyAsync(h->runs, runs.data(), runs.size() * sizeof(int64_t),
                                  cudaMemcpyHostToDevice, ctx->stream));
    if (h->xfull) {
      const size_t es = elem_size(h->dtype);
      GB_CHECK_CUDA(cudaMemsetAsync(h->xfull, 0, (size_t)h->xnumel * es, ctx->stream));
      h->xcomp = dalloc(h, (size_t)h->ncompact * es);  // follows the new compact length
    }
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  if (!h->aa_glc || h->kJ.empty()) {  // no fused chain: nothing more to restrict
    grouped_prepare(h);
    return;
  }
  GB_REQUIRE(h->aa_Dl == Dl && h->aa_Dr == Dr, "set_sectors: bond dimensions");
  const int64_t chr = h->aa_chr;
  // fused physical charges of the mix rows
  std::vector<int> qp(h->aa_np);
  if (h->kind == GB_HEFF_AC2) {
    const int64_t d1 = h->xdims[1], d2 = h->xdims[3];
    GB_REQUIRE(qp2, "set_sectors: two physical legs expected");
    for (int64_t sb = 0; sb < d2; ++sb)
      for (int64_t sa = 0; sa < d1; ++sa) qp[sa + d1 * sb] = qp1[sa] + qp2[sb];
  } else {
    for (int64_t s = 0; s < h->aa_np; ++s) qp[s] = qp1[s];
  }
  // channel charges from GL itself
  int* dev = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(&dev, (Dl + chr + 1) * sizeof(int), ctx->stream));
  std::vector<int> init(chr + 1, INT_MIN);
  init[chr] = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(dev, ql, Dl * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  GB_CHECK_CUDA(cudaMemcpyAsync(dev + Dl, init.data(), (chr + 1) * sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
  channel_charge_kernel<<<(unsigned)std::min<int64_t>((Dl * Dl * chr + 255) / 256, 152 * 16),
                          256, 0, ctx->stream>>>((const double*)h->aa_glc, Dl, chr,
                                                 is_cplx(h->dtype) ? 1 : 0, dev, dev + Dl,
                                                 dev + Dl + chr);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
  std::vector<int> dq(chr + 1);
  GB_CHECK_CUDA(cudaMemcpyAsync(dq.data(), dev + Dl, (chr + 1) * sizeof(int),
                                cudaMemcpyDeviceToHost, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  GB_CHECK_CUDA(cudaFreeAsync(dev, ctx->stream));
  GB_REQUIRE(dq[chr] == 0, "set_sectors: the left environment does not conserve these charges");
  const int64_t nJ = (int64_t)h->kJ.size();
  std::vector<int2> tab((size_t)nJ * Dr);
  int64_t mx = 0;
  for (int64_t n = 0; n < Dr; ++n)
    for (int64_t J = 0; J < nJ; ++J) {
      int2 r{0, 0};
      const int d = dq[h->Jc[J]];
      if (d != INT_MIN) r = sector((int64_t)qr[n] - d - qp[h->Jp[J]]);
      tab[(size_t)n * nJ + J] = r;
      mx = std::max<int64_t>(mx, r.y - r.x);
    }
  if (!h->arange) h->arange = (int2*)dalloc(h, tab.size() * sizeof(int2));
  GB_CHECK_CUDA(cudaMemcpyAsync(h->arange, tab.data(), tab.size() * sizeof(int2),
                                cudaMemcpyHostToDevice, ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  h->arange_max = mx;
  h->lam_J.assign(nJ, INT64_MIN);
  for (int64_t J = 0; J < nJ; ++J)
    if (dq[h->Jc[J]] != INT_MIN) h->lam_J[J] = (int64_t)dq[h->Jc[J]] + qp[h->Jp[J]];
  h->dq_l.assign(dq.begin(), dq.begin() + chr);
  h->arange_h = std::move(tab);
  grouped_prepare(h);
}

// ------------------------------------------------------------------ grouped sector blocks
// dq[j] = q_r(r) - q_r(r') over the nonzero entries of GR's continuing channel j (layout
// (r', j, r)); INT_MIN: the channel is zero
__global__ void channel_charge_grc_kernel(const double* __restrict__ grc, int64_t Dr, int64_t chc,
                                          const int* __restrict__ qr, int* dq, int* bad) {
  const int64_t n = Dr * chc * Dr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (grc[i] == 0.0) continue;
    const int64_t rp = i % Dr, j = (i / Dr) % chc, r = i / (Dr * chc);
    const int v = qr[r] - qr[rp];
    int cur = *(volatile int*)&dq[j];
    if (cur == INT_MIN) {
      cur = atomicCAS(&dq[j], INT_MIN, v);
      if (cur == INT_MIN) cur = v;
    }
    if (cur != v) atomicExch(bad, 1);
  }
}

static gb::LegSpec leg(int64_t n, int which, int sign = 1) {
  gb::LegSpec l;
  l.n = n;
  l.which = which;
  l.sign = sign;
  return l;
}

// charge labels of every GEMM step's M, K and N index (the vector x is allowed where
// q_l + q_s1 (+ q_s2) = q_r; continuing channels carry the charge they add to the bond);
// false when a step has no labelling (the grouped form is then not used)
static bool assign_legs(gb_heff* h) {
  using namespace gb;
  const bool two = h->kind == GB_HEFF_AC2;
  const int64_t Dl = h->xdims[0], d1 = h->xdims[1], Dr = h->xdims[2], d2 = two ? h->xdims[3] : 1;
  const LegSpec L = leg(Dl, Q_L), R = leg(Dr, Q_R), P1 = leg(d1, Q_P1), P1m = leg(d1, Q_P1, -1),
                P2 = leg(d2, Q_P2), P2m = leg(d2, Q_P2, -1);
  const LegSpec CL = leg(h->aa_chr, Q_CL), CRm = leg(h->aa_chc, Q_CR, -1);
  const std::vector<LegSpec> left = two ? std::vector<LegSpec>{L, P1, P2}
                                        : std::vector<LegSpec>{L, P1};   // (l s1 s2)
  const std::vector<LegSpec> right = two ? std::vector<LegSpec>{P1m, P2m, R}
                                         : std::vector<LegSpec>{P1m, R};  // (s1 s2 r)
  for (Step& st : h->steps) {
    if (!st.is_gemm) continue;
    const std::string& n = st.name;
    if (n == "AA1" || n == "A1") {  // T1[(l' s'), (c' r)] = X[(l' s'), r'] GRc[r', (c' r)]
      st.lM = left; st.lK = {R}; st.lN = {CRm, R};
    } else if (n == "AA3" || n == "A3") {  // Y[l, (s r)] += GLc[l, (l' c)] T2[(l' c), (s r)]
      st.lM = {L}; st.lK = {L, CL}; st.lN = right;
    } else if (n == "CA" || n == "C") {  // Y[l, (s r)] += X[l, (s' r')] M[(s' r'), (s r)]
      st.lM = {L}; st.lK = right; st.lN = right;
    } else if (n == "AB" || n == "B") {  // Y[(l s), r] += M[(l s), (l' s')] X[(l' s'), r]
      st.lM = left; st.lK = left; st.lN = {R};
    } else if (n == "IC") {  // Y[(l s1), (s2 r)] += X[(l s1), (s2' r')] M
      st.lM = {L, P1}; st.lK = {P2m, R}; st.lN = {P2m, R};
    } else if (n == "BE") {  // Y[(l s1), (s2 r)] += M[(l s1), (l' s1')] X
      st.lM = {L, P1}; st.lK = {L, P1}; st.lN = {P2m, R};
    } else if (n == "II" || n == "I") {  // Y[(l s), r] += X[(l s), r'] GR[r', 0, r]
      st.lM = left; st.lK = {R}; st.lN = {R};
    } else if (n == "EE" || n == "E") {  // Y[l, (s r)] += GL[l, l', end] X[l', (s r)]
      st.lM = {L}; st.lK = {L}; st.lN = right;
    } else {
      return false;
    }
  }
  return true;
}

// Plans, packed constant operands and the mix table of the grouped form.  Every constant
// operand is checked to lie inside its blocks (nonzero count of the packed blocks equal to
// that of the dense operand): an operator that does not conserve the given charges is an
// error, never silently truncated.
static void grouped_prepare(gb_heff* h) {
  using namespace gb;
  gb_ctx* ctx = h->ctx;
  h->gp_ready = false;
  if (h->sched != GB_SCHED_GROUPED || h->prec == GB_PREC_FP64 || is_cplx(h->dtype) ||
      !h->runs || h->kind == GB_HEFF_C)
    return;
  if (!assign_legs(h)) return;
  const bool chain = h->aa_glc && !h->kJ.empty();
  if (chain) {
    GB_REQUIRE((int64_t)h->dq_l.size() == h->aa_chr && !h->arange_h.empty(),
               "grouped: sectors of the fused chain missing");
    // continuing-channel charges of GR, read off GR itself
    const int64_t Dr = h->xdims[2], chc = h->aa_chc;
    int* dev = nullptr;
    GB_CHECK_CUDA(cudaMallocAsync(&dev, (Dr + chc + 1) * sizeof(int), ctx->stream));
    std::vector<int> init(chc + 1, INT_MIN);
    init[chc] = 0;
    GB_CHECK_CUDA(cudaMemcpyAsync(dev, h->q_r.data(), Dr * sizeof(int), cudaMemcpyHostToDevice,
                                  ctx->stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(dev + Dr, init.data(), (chc + 1) * sizeof(int),
                                  cudaMemcpyHostToDevice, ctx->stream));
    channel_charge_grc_kernel<<<(unsigned)std::min<int64_t>((Dr * chc * Dr + 255) / 256,
                                                            152 * 16),
                                256, 0, ctx->stream>>>((const double*)h->aa_grc, Dr, chc, dev,
                                                       dev + Dr, dev + Dr + chc);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    std::vector<int> dq(chc + 1);
    GB_CHECK_CUDA(cudaMemcpyAsync(dq.data(), dev + Dr, (chc + 1) * sizeof(int),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    GB_CHECK_CUDA(cudaFreeAsync(dev, ctx->stream));
    GB_REQUIRE(dq[chc] == 0, "grouped: the right environment does not conserve these charges");
    h->dq_r.assign(dq.begin(), dq.begin() + chc);
  }
  std::vector<const int32_t*> q(Q_COUNT, nullptr);
  q[Q_L] = h->q_l.data();
  q[Q_R] = h->q_r.data();
  q[Q_P1] = h->q_p1.data();
  q[Q_P2] = h->q_p2.empty() ? nullptr : h->q_p2.data();
  q[Q_CL] = h->dq_l.empty() ? nullptr : h->dq_l.data();
  q[Q_CR] = h->dq_r.empty() ? nullptr : h->dq_r.data();
  auto alloc = [h](size_t b) { return dalloc(h, b); };
  h->gsteps.assign(h->steps.size(), GStep());
  h->t2_step = -1;
  // the term X . M with the chain's last GEMM's output blocks (CA for AC2, C for AC) runs
  // inside that GEMM: both are Y[l, (s r)] (+)= A[l, k] B[k, (s r)], so their K spaces stack
  // (GLc | X) . (T2 ; M) and Y is written once
  h->merged_into.assign(h->steps.size(), -1);
  h->merged_k.assign(h->steps.size(), 0);
  {
    int i3 = -1, ic = -1;
    for (size_t i = 0; i < h->steps.size(); ++i) {
      const Step& st = h->steps[i];
      if (st.is_gemm && st.t2_consumer) i3 = (int)i;
      if (st.is_gemm && (st.name == "CA" || st.name == "C") && st.srcA == S_X &&
          st.srcB == S_CONST && st.dst == S_Y)
        ic = (int)i;
    }
    if (i3 >= 0 && ic > i3) {
      const Step &a = h->steps[i3], &c = h->steps[ic];
      if (a.dst == S_Y && a.M == c.M && a.N == c.N && a.ldc == c.ldc && c.accumulate &&
          a.opA == 'N' && a.opB == 'N' && c.opA == 'N' && c.opB == 'N') {
        h->merged_into[ic] = i3;
        h->merged_k[i3] = a.K;
      }
    }
  }
  for (size_t i = 0; i < h->steps.size(); ++i) {
    const Step& st = h->steps[i];
    if (!st.is_gemm || h->merged_into[i] >= 0) continue;
    GB_REQUIRE(st.opA == 'N' && st.opB == 'N', "grouped: transposed operands");
    const std::vector<int32_t> lM = leg_labels(st.lM, q), lN = leg_labels(st.lN, q);
    std::vector<int32_t> lK = leg_labels(st.lK, q);
    GB_REQUIRE((int64_t)lM.size() == st.M && (int64_t)lK.size() == st.K &&
                   (int64_t)lN.size() == st.N,
               "grouped: labels do not match the GEMM shape of step " + st.name);
    const Step* mc = nullptr;  // the merged step, if any
    std::vector<int32_t> lKc;
    for (size_t j = 0; j < h->steps.size(); ++j)
      if (h->merged_into[j] == (int)i) mc = &h->steps[j];
    if (mc) {
      lKc = leg_labels(mc->lK, q);
      GB_REQUIRE((int64_t)lKc.size() == mc->K, "grouped: labels of the merged step");
      lK.insert(lK.end(), lKc.begin(), lKc.end());
    }
    GStep& gs = h->gsteps[i];
    gplan_build(gs.plan, lM, lK, lN, !st.accumulate, st.ldc, std::max(1, ctx->num_sms));
    gplan_upload(ctx, gs.plan, alloc);
    for (int sd = 0; sd < 2; ++sd)
      goperand_init(ctx, gs.op[sd], gs.plan, sd, dalloc(h, goperand_bytes(gs.plan, sd, h->prec)),
                    h->prec);
    // constants: original A(m, k) at m + lda k, original B(k, n) at k + ldb n.  A nonzero
    // whose row and column labels differ would be dropped by the blocks: refuse it (entries
    // of a conserved label that has no group on the other side of the GEMM meet only zeros
    // of x and are dropped rightly)
    const std::vector<int32_t> lKs(lK.begin(), lK.begin() + st.K);  // this step's own K
    const int64_t kown = mc ? st.K : INT64_MAX;
    if (st.srcA == S_CONST) {
      GB_REQUIRE(label_violations(ctx, (const double*)st.cA, st.M, st.K, 1, st.lda, lM, lKs) == 0,
                 "grouped: operator term " + st.name + " does not conserve the given charges");
      gpack(ctx, gs.plan, 0, (const double*)st.cA, 1, st.lda, gs.op[0], false, 0, kown);
    }
    if (st.srcB == S_CONST) {
      GB_REQUIRE(label_violations(ctx, (const double*)st.cB, st.N, st.K, st.ldb, 1, lN, lKs) == 0,
                 "grouped: operator term " + st.name + " does not conserve the given charges");
      gpack(ctx, gs.plan, 1, (const double*)st.cB, st.ldb, 1, gs.op[1], false, 0, kown);
    }
    if (mc) {
      // the merged step's constant B at K offset st.K (its A is x, packed every apply)
      GB_REQUIRE(mc->srcB == S_CONST && mc->srcA == S_X, "grouped: merged step operands");
      GB_REQUIRE(label_violations(ctx, (const double*)mc->cB, mc->N, mc->K, mc->ldb, 1, lN,
                                  lKc) == 0,
                 "grouped: operator term " + mc->name + " does not conserve the given charges");
      gpack(ctx, gs.plan, 1, (const double*)mc->cB, mc->ldb, 1, gs.op[1], false, st.K,
            st.K + mc->K);
    }
    if (st.t2_consumer) {
      GB_REQUIRE(st.srcB == S_T2, "grouped: T2 is the B operand of its consumer");
      h->t2_step = (int)i;
    }
  }
  if (chain) {
    GB_REQUIRE(h->t2_step >= 0, "grouped: the fused chain has no consumer");
    const GPlan& P = h->gsteps[h->t2_step].plan;
    // packed row of every dense N index, position of every dense K index within its group
    std::vector<int32_t> posN(h->t2N, -1), kpos(h->t2K, -1), ngrp(h->t2N, -1), kgrp(h->t2K, -1);
    for (int g = 0; g < P.G; ++g) {
      for (int32_t r = P.side[1].gstart[g]; r < P.side[1].gstart[g + 1]; ++r) {
        posN[P.side[1].dense[r]] = r;
        ngrp[P.side[1].dense[r]] = g;
      }
      for (int32_t k = P.kstart[g]; k < P.kstart[g + 1]; ++k) {
        // K members past T2's rows belong to a term stacked along K (its x . M part)
        if (P.kdense[k] >= h->t2K) continue;
        kpos[P.kdense[k]] = k - P.kstart[g];
        kgrp[P.kdense[k]] = g;
      }
    }
    const int64_t nJ = (int64_t)h->kJ.size(), Dr = h->xdims[2];
    std::vector<GMixEntry> ent((size_t)nJ * Dr);
    for (int64_t n = 0; n < Dr; ++n)
      for (int64_t J = 0; J < nJ; ++J) {
        const int2 ar = h->arange_h[(size_t)n * nJ + J];
        GMixEntry e{ar.x, ar.y, -1, 0};
        if (ar.y > ar.x) {
          const int64_t m = h->mJ[J] + n * h->mn;
          const int64_t k0 = ar.x + h->kJ[J], k1 = ar.y - 1 + h->kJ[J];
          // a row or contraction index outside every block of the consumer meets only
          // zeros there (its charge has no partner on the other side): nothing to write
          if (posN[m] >= 0 && kpos[k0] >= 0) {
            e.row = posN[m];
            e.kst = kpos[k0];
            GB_REQUIRE(ngrp[m] == kgrp[k0] && kgrp[k1] == kgrp[k0] &&
                           kpos[k1] == e.kst + (ar.y - 1 - ar.x),
                       "grouped: the fused chain's sectors do not match its consumer's blocks");
          }
        }
        ent[(size_t)n * nJ + J] = e;
      }
    h->gmix = (GMixEntry*)dalloc(h, ent.size() * sizeof(GMixEntry));
    GB_CHECK_CUDA(cudaMemcpyAsync(h->gmix, ent.data(), ent.size() * sizeof(GMixEntry),
                                  cudaMemcpyHostToDevice, ctx->stream));
    build_staged_mix(h, Dr);
    // T1 is read only inside its blocks; the entries no block writes stay zero
    GB_REQUIRE(h->t1, "grouped: T1 buffer missing");
    GB_CHECK_CUDA(cudaMemsetAsync(h->t1, 0, (size_t)h->t1_elems * elem_size(h->dtype),
                                  ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  h->gp_prec = h->prec;
  h->gp_ready = true;
}

// The staged form of the chain mix (gmix_staged_run): rows J of one charge form a group
// whose input range is the same at every column; each group stages the inputs its rows
// read.  Left unbuilt (the plain gmix_run is used) when a group's inputs do not fit the
// staging buffer.
static void build_staged_mix(gb_heff* h, int64_t Dr) {
  using namespace gb;
  h->gmix_st = GMixStaged();
  const Step* mixstep = nullptr;
  for (const Step& s : h->steps)
    if (s.t2_producer) mixstep = &s;
  if (!mixstep || h->lam_J.empty()) return;
  const MixPlan& mp = mixstep->mixh;
  const int64_t nJ = (int64_t)h->kJ.size();
  if ((int64_t)mp.row_ptr.size() != nJ + 1 || (int64_t)h->lam_J.size() != nJ) return;
  std::map<int64_t, std::vector<int>> byq;
  for (int64_t J = 0; J < nJ; ++J)
    if (h->lam_J[J] != INT64_MIN) byq[h->lam_J[J]].push_back((int)J);
  const int NL = (int)byq.size();
  if (NL == 0) return;
  std::vector<int> jlist, jstart{0}, ilist, istart{0}, rp, rstart, li, cstart{0};
  std::vector<float> vh, vl;  // per group: its rows' entries (local input, coefficient hi + lo)
  std::vector<int2> rng((size_t)Dr * NL);
  size_t max_ni = 0, max_csr = 0, max_csr_tf = 0;
  int g = 0;
  for (const auto& kv : byq) {
    const std::vector<int>& Js = kv.second;
    std::vector<int> ins;
    for (int J : Js)
      for (int e = mp.row_ptr[J]; e < mp.row_ptr[J + 1]; ++e) ins.push_back(mp.col[e]);
    std::sort(ins.begin(), ins.end());
    ins.erase(std::unique(ins.begin(), ins.end()), ins.end());
    const size_t ni = ins.size();
    rstart.push_back((int)rp.size());
    for (int J : Js) {
      rp.push_back((int)li.size());
      for (int e = mp.row_ptr[J]; e < mp.row_ptr[J + 1]; ++e) {
        li.push_back((int)(std::lower_bound(ins.begin(), ins.end(), mp.col[e]) - ins.begin()));
        const float h = (float)mp.val[e];
        vh.push_back(h);
        vl.push_back((float)(mp.val[e] - (double)h));
      }
    }
    rp.push_back((int)li.size());
    cstart.push_back((int)li.size());
    // one input range per (column, group): every row of the group must agree
    for (int64_t n = 0; n < Dr; ++n) {
      const int2 r0 = h->arange_h[(size_t)n * nJ + Js[0]];
      for (int J : Js) {
        const int2 r = h->arange_h[(size_t)n * nJ + J];
        if (r.x != r0.x || r.y != r0.y) return;
      }
      rng[(size_t)n * NL + g] = r0;
    }
    jlist.insert(jlist.end(), Js.begin(), Js.end());
    jstart.push_back((int)jlist.size());
    ilist.insert(ilist.end(), ins.begin(), ins.end());
    istart.push_back((int)ilist.size());
    const size_t ne = (size_t)(cstart[g + 1] - cstart[g]);
    max_ni = std::max(max_ni, ni);
    max_csr = std::max(max_csr, Js.size() + 1 + 2 * ne);        // rows, index, hi
    max_csr_tf = std::max(max_csr_tf, Js.size() + 1 + 3 * ne);  // + lo
    ++g;
  }
  // shared memory: the rows' entries plus a chunk of inputs
  const int64_t cap = 96 * 1024 / 4;  // words
  const int64_t amax = std::max<int64_t>(h->arange_max, 1);
  auto chunk_for = [&](int64_t words) -> int64_t {
    // the inputs' base offsets (int64 each, 8-byte aligned) follow the staged chunk
    const int64_t room = cap - words - 2 * (int64_t)max_ni - 4;
    if (room <= 0) return 0;
    return std::min<int64_t>(amax, room / (int64_t)std::max<size_t>(max_ni, 1));
  };
  // the staged inputs start 16-byte aligned after the entries
  max_csr = (max_csr + 3) / 4 * 4;
  max_csr_tf = (max_csr_tf + 3) / 4 * 4;
  const int64_t chunk = chunk_for((int64_t)max_csr), chunk_tf = chunk_for((int64_t)max_csr_tf);
  if ((chunk < 32 && chunk < amax) || (chunk_tf < 32 && chunk_tf < amax) || chunk < 1 ||
      chunk_tf < 1)
    return;
  // one device blob for the tables
  std::vector<char> blob;
  auto put = [&](const void* src, size_t bytes) {
    const size_t off = (blob.size() + 255) / 256 * 256;
    blob.resize(off + std::max<size_t>(bytes, 16), 0);
    if (bytes) memcpy(blob.data() + off, src, bytes);
    return off;
  };
  const size_t o_r = put(rng.data(), rng.size() * sizeof(int2));
  const size_t o_jl = put(jlist.data(), jlist.size() * 4), o_js = put(jstart.data(), jstart.size() * 4);
  const size_t o_il = put(ilist.data(), ilist.size() * 4), o_is = put(istart.data(), istart.size() * 4);
  const size_t o_rp = put(rp.data(), rp.size() * 4), o_rs = put(rstart.data(), rstart.size() * 4);
  const size_t o_li = put(li.data(), li.size() * 4), o_cs = put(cstart.data(), cstart.size() * 4);
  const size_t o_vh = put(vh.data(), vh.size() * 4), o_vl = put(vl.data(), vl.size() * 4);
  char* d = (char*)dalloc(h, blob.size());
  GB_CHECK_CUDA(cudaMemcpyAsync(d, blob.data(), blob.size(), cudaMemcpyHostToDevice,
                                h->ctx->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(h->ctx->stream));
  GMixStaged& st = h->gmix_st;
  st.rng = (const int2*)(d + o_r);
  st.jlist = (const int*)(d + o_jl);
  st.jstart = (const int*)(d + o_js);
  st.ilist = (const int*)(d + o_il);
  st.istart = (const int*)(d + o_is);
  st.rp = (const int*)(d + o_rp);
  st.rstart = (const int*)(d + o_rs);
  st.li = (const int*)(d + o_li);
  st.cstart = (const int*)(d + o_cs);
  st.vh = (const float*)(d + o_vh);
  st.vl = (const float*)(d + o_vl);
  st.chunk = (int)chunk;
  st.chunk_tf32 = (int)chunk_tf;
  st.nnz_per_row = jlist.empty() ? 0.0 : (double)li.size() / (double)jlist.size();
  st.csr_floats = (int)max_csr;
  st.csr_floats_tf32 = (int)max_csr_tf;
  st.smem = (size_t)(st.csr_floats + chunk * max_ni + 1) * 4 + (size_t)max_ni * 8;
  st.smem_tf32 = (size_t)(st.csr_floats_tf32 + chunk_tf * max_ni + 1) * 4 + (size_t)max_ni * 8;
  st.NL = NL;
}

// y = H x through the grouped plans.  x: dense embedding, zero outside the sectors; every
// allowed entry of y is written (the first GEMM into y overwrites, the rest accumulate);
// entries outside the sectors are zeroed only when y is not the operator's own staging
// vector (whose outside entries are never read).
static void heff_apply_grouped(gb_heff* h, const void* x, void* y) {
  using namespace gb;
  gb_ctx* ctx = h->ctx;
  if (h->y_zero_first || y != h->yfull) fill_zero(ctx, y, (size_t)h->xnumel * elem_size(h->dtype));
  for (size_t i = 0; i < h->steps.size(); ++i) {
    const Step& st = h->steps[i];
    if (st.is_gemm && h->merged_into[i] >= 0) continue;  // runs inside its carrier's GEMM
    if (st.is_gemm) {
      GStep& gs = h->gsteps[i];
      const int64_t kown = h->merged_k[i] ? st.K : INT64_MAX;
      if (st.srcA == S_X) gpack(ctx, gs.plan, 0, (const double*)x, 1, st.lda, gs.op[0], false, 0, kown);
      if (st.srcB == S_X) gpack(ctx, gs.plan, 1, (const double*)x, st.ldb, 1, gs.op[1], false, 0, kown);
      if (h->merged_k[i])
        for (size_t j = 0; j < h->steps.size(); ++j)
          if (h->merged_into[j] == (int)i)  // the merged term's x . M: A = x at K offset st.K
            gpack(ctx, gs.plan, 0, (const double*)x, 1, h->steps[j].lda, gs.op[0], false, st.K,
                  st.K + h->steps[j].K);
      const bool t1 = st.dst == S_T1;
      gemm_grouped(ctx, gs.plan, gs.op[0], gs.op[1], 1.0, st.accumulate ? 1.0 : 0.0,
                   t1 ? h->t1 : y, t1);
      if (ctx->counting) gcount_products(ctx, gs.plan, gs.op[0], gs.op[1]);
    } else if (st.t2_producer) {
      const bool staged = h->gmix_st.NL > 0 &&
                          (ctx->staged_mix == 2 ||
                           (ctx->staged_mix == 1 && h->gmix_st.nnz_per_row >= 4.0));
      if (staged)
        gmix_staged_run(ctx, st.mix, h->gmix_st, h->gmix, (const float*)h->t1,
                        h->gsteps[h->t2_step].op[1]);
      else
        gmix_run(ctx, st.mix, h->gmix, h->arange_max, (const float*)h->t1,
                 h->gsteps[h->t2_step].op[1]);
    } else {
      GB_REQUIRE(st.src == S_X && st.dst == S_Y, "grouped: unexpected mix step");
      mix_run(ctx, st.mix, h->dtype, x, y, st.accumulate ? 1.0 : 0.0);
    }
  }
}

static void ensure_prepacked(gb_heff* h) {
  if (h->prepacked) return;
  for (auto& st : h->steps)
    if (st.is_gemm) prepack(h, st);
  h->prepacked = true;
}

void heff_set_precision(gb_heff* h, int prec) {
  GB_REQUIRE(prec == GB_PREC_FP64 || prec == GB_PREC_BF16X3 || prec == GB_PREC_TF32X3,
             "heff: precision");
  if (prec != h->prec) {
    // packed constants and the packed T2 follow the plane type; repack on change (the old
    // buffers stay owned by the operator until it is freed)
    for (auto& s : h->steps) s.hasPA = s.hasPB = false;
    h->t2p_ready = false;
    h->prepacked = false;
    h->prec = prec;
    if (h->runs) grouped_prepare(h);  // the grouped form follows the plane type too
  }
  h->prec = prec;
  if (!h->gp_ready) ensure_prepacked(h);
}

// y = H x (device pointers, device layout)
void heff_apply_raw(gb_heff* h, const void* x, void* y) {
  gb_ctx* ctx = h->ctx;
  if (h->gp_ready && h->gp_prec == h->prec) {
    heff_apply_grouped(h, x, y);
    return;
  }
  ensure_prepacked(h);
  if (h->y_zero_first) fill_zero(ctx, y, (size_t)h->xnumel * elem_size(h->dtype));
  auto ptr = [&](int src, const void* c) -> const void* {
    switch (src) {
      case S_CONST: return c;
      case S_X: return x;
      case S_Y: return y;
      case S_T1: return h->t1;
      case S_T2: return h->t2;
    }
    return nullptr;
  };
  const bool fused_t2 = h->prec != GB_PREC_FP64 && h->t2p_ready;
  if (!fused_t2 && h->t2_elems && !h->t2)
    h->t2 = dalloc(h, (size_t)h->t2_elems * elem_size(h->dtype));
  for (const Step& s : h->steps) {
    if (s.is_gemm) {
      void* C = (void*)ptr(s.dst, nullptr);
      double beta = s.accumulate ? 1.0 : 0.0;
      const Packed* pB = s.hasPB ? &s.pB : nullptr;
      if (fused_t2 && s.t2_consumer) pB = &h->t2p;
      uint32_t* omap = (fused_t2 && s.dst == S_T1 && h->t1map) ? h->t1map : nullptr;
      // T1 of the fused chain is written as the FP32 accumulator itself (exact: alpha = 1,
      // beta = 0) and read back by the fused mix: half the traffic of the largest
      // intermediate
      const bool f32 = omap != nullptr && !s.accumulate;
      gemm(ctx, h->prec, h->dtype, s.opA, s.opB, s.M, s.N, s.K, 1.0, ptr(s.srcA, s.cA), s.lda, 0,
           ptr(s.srcB, s.cB), s.ldb, 0, beta, C, s.ldc, 0, 1, s.hasPA ? &s.pA : nullptr, pB,
           omap, f32);
      if (omap) h->t1_f32 = f32;
    } else if (fused_t2 && s.t2_producer) {
      const int64_t* kJ = (const int64_t*)h->kmJ_dev;
      MixSkipDev sk;
      if (h->t1map && s.src == S_T1) {
        sk.xmap = h->t1map;
        sk.onc = (h->t1N + 127) / 128;
        sk.roff = h->t1rc_dev;
        sk.coff = h->t1rc_dev + h->t1roff.size();
        sk.xnM = h->t1xnM;
        sk.prev = h->t2prev;
      }
      if (h->arange && s.src == S_T1) {
        sk.arange = h->arange;
        sk.arange_max = h->arange_max;
      }
      mixpack_run(ctx, s.mix, kJ, kJ + h->kJ.size(), h->mn, h->dtype, ptr(s.src, nullptr), h->t2p,
                  h->t2K, h->t2N, sk.xmap ? &sk : nullptr, sk.xmap && h->t1_f32);
    } else {
      mix_run(ctx, s.mix, h->dtype, ptr(s.src, nullptr), (void*)ptr(s.dst, nullptr),
              s.accumulate ? 1.0 : 0.0);
    }
  }
}

}  // namespace gb

namespace gb {
struct HeffInfo {
  gb_ctx* ctx;
  int kind, dtype, prec, xndim;
  int64_t xdims[4];
  int64_t xnumel;
  double flops;
  const char* terms;
};
// one line per contraction step: its shape and, for a grouped sector-block GEMM, the plan
// (groups, tiles, K-blocks of the longest tile, tile work over nonzero block work)
std::string heff_describe(const gb_heff* h) {
  std::ostringstream os;
  for (size_t i = 0; i < h->steps.size(); ++i) {
    const Step& s = h->steps[i];
    os << s.name << (s.is_gemm ? " gemm" : " mix");
    if (s.is_gemm) os << " M=" << s.M << " N=" << s.N << " K=" << s.K;
    if (i < h->merged_into.size() && h->merged_into[i] >= 0)
      os << " (stacked along K into " << h->steps[h->merged_into[i]].name << ")";
    if (i < h->gsteps.size() && !h->gsteps[i].plan.tiles.empty()) {
      const GPlan& p = h->gsteps[i].plan;
      int64_t maxkb = 0, kb = 0;
      for (const GTile& t : p.tiles) {
        maxkb = std::max<int64_t>(maxkb, t.nkb);
        kb += t.nkb;
      }
      os << " grouped G=" << p.G << " units=" << p.tiles.size()
         << " split_tiles=" << p.ncounters << " kblocks=" << kb
         << " max_unit_kblocks=" << maxkb << " trans=" << (p.trans ? 1 : 0)
         << " block_gflop=" << p.block_flops * 1e-9 << " tile_gflop=" << p.tile_flops * 1e-9;
    }
    os << "\n";
  }
  return os.str();
}

HeffInfo heff_info(const gb_heff* h) {
  HeffInfo hi;
  hi.ctx = h->ctx;
  hi.kind = h->kind;
  hi.dtype = h->dtype;
  hi.prec = h->prec;
  hi.xndim = h->xndim;
  for (int i = 0; i < 4; ++i) hi.xdims[i] = h->xdims[i];
  hi.xnumel = h->xnumel;
  hi.flops = h->flops;
  hi.terms = h->terms.c_str();
  return hi;
}
}  // namespace gb
