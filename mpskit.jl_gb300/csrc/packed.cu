// Tile-packed storage of block-sparse tensors (environments of U(1) states).
//
// A charge-conserving environment GL[a, a', w] held in the charge-sorted dense embedding is
// zero outside one shifted block diagonal per channel: at D = 2048 with ~33 sectors about a
// tenth of its 64 x 64 tiles hold a nonzero.  gb_tensor_pack keeps only those tiles (exactly:
// a tile is dropped only if every element is +-0.0), gb_packed_unpack rebuilds the dense
// embedding (zeros elsewhere), so FiniteEnvironments can keep every environment of a sweep
// resident (the reference's cache, src/environments/finite_envs.jl:110-151) in a tenth of the
// memory and expand the two it is using.  The storage is charge-agnostic: the tiles are
// found by scanning, so any tensor whose zeros come in tile-sized blocks packs well.
//
// Matrix view: rows = first device dimension, columns = the product of the others; tiles of
// PT x PT elements, stored column-major one after the other in increasing tile order.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "gb_common.h"

struct gb_packed {
  gb_ctx* ctx = nullptr;
  int kind = 0, dtype = 0, ndim = 0;
  int64_t dims[6] = {0, 0, 0, 0, 0, 0};
  int64_t rows = 0, cols = 0;
  int64_t nkept = 0;           // stored tiles
  int64_t* d_tiles = nullptr;  // tile index (tr + ntr * tc) of every stored tile
  void* d_data = nullptr;      // [nkept][PT * PT] elements
  size_t bytes = 0;
};

namespace gb {
namespace {
constexpr int PT = 64;

inline int64_t dev_rows(const gb_tensor* t) {
  // first dimension of the device layout (see include/mpsgb.h): GR is (b', w, b), the
  // others start with their first reference leg
  return t->dims[0];
}

// one warp per tile: 1 if any element of the tile is nonzero
__global__ void tile_flags_kernel(const unsigned long long* __restrict__ src, int64_t rows,
                                  int64_t cols, int64_t ntr, int64_t ntiles, int words,
                                  unsigned char* __restrict__ flag) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntiles) return;
  const int64_t tr = warp % ntr, tc = warp / ntr;
  const int64_t r0 = tr * PT, c0 = tc * PT;
  const int64_t nr = min((int64_t)PT, rows - r0), nc = min((int64_t)PT, cols - c0);
  bool nz = false;
  for (int64_t c = 0; c < nc && !nz; ++c) {
    const unsigned long long* col = src + ((c0 + c) * rows + r0) * words;
    for (int64_t i = lane; i < nr * words; i += 32) nz |= (col[i] << 1) != 0ull;  // +-0.0 are zero
    nz = __any_sync(0xffffffffu, nz);
  }
  if (lane == 0) flag[warp] = nz ? 1 : 0;
}

// pack (dir = 0) or unpack (dir = 1) the listed tiles: one block per stored tile
__global__ void tile_copy_kernel(unsigned long long* __restrict__ dense,
                                 unsigned long long* __restrict__ packed,
                                 const int64_t* __restrict__ tiles, int64_t rows, int64_t cols,
                                 int64_t ntr, int words, int dir) {
  const int64_t k = blockIdx.x;
  const int64_t t = tiles[k];
  const int64_t r0 = (t % ntr) * PT, c0 = (t / ntr) * PT;
  const int64_t nr = min((int64_t)PT, rows - r0), nc = min((int64_t)PT, cols - c0);
  unsigned long long* tile = packed + k * (int64_t)PT * PT * words;
  for (int64_t c = threadIdx.y; c < nc; c += blockDim.y) {
    unsigned long long* col = dense + ((c0 + c) * rows + r0) * words;
    unsigned long long* tc = tile + c * PT * words;
    for (int64_t i = threadIdx.x; i < nr * words; i += blockDim.x) {
      if (dir == 0) tc[i] = col[i];
      else col[i] = tc[i];
    }
  }
}
}  // namespace

gb_packed* tensor_pack(gb_ctx* ctx, const gb_tensor* t) {
  const int words = elem_size(t->dtype) / 8;
  const int64_t rows = dev_rows(t), n = numel(t);
  const int64_t cols = rows ? n / rows : 0;
  const int64_t ntr = (rows + PT - 1) / PT, ntc = (cols + PT - 1) / PT, nt = ntr * ntc;
  gb_packed* p = new gb_packed();
  p->ctx = ctx;
  p->kind = t->kind;
  p->dtype = t->dtype;
  p->ndim = t->ndim;
  for (int i = 0; i < 6; ++i) p->dims[i] = t->dims[i];
  p->rows = rows;
  p->cols = cols;
  if (nt == 0) return p;
  try {
    unsigned char* dflag = nullptr;
    GB_CHECK_CUDA(cudaMallocAsync(&dflag, nt, ctx->stream));
    tile_flags_kernel<<<(unsigned)((nt * 32 + 255) / 256), 256, 0, ctx->stream>>>(
        (const unsigned long long*)t->data, rows, cols, ntr, nt, words, dflag);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    std::vector<unsigned char> flag(nt);
    GB_CHECK_CUDA(cudaMemcpyAsync(flag.data(), dflag, nt, cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaFreeAsync(dflag, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<int64_t> kept;
    for (int64_t i = 0; i < nt; ++i)
      if (flag[i]) kept.push_back(i);
    p->nkept = (int64_t)kept.size();
    if (p->nkept == 0) return p;
    p->bytes = (size_t)p->nkept * PT * PT * elem_size(t->dtype);
    GB_CHECK_CUDA(cudaMallocAsync(&p->d_tiles, kept.size() * sizeof(int64_t), ctx->stream));
    GB_CHECK_CUDA(cudaMallocAsync(&p->d_data, p->bytes, ctx->stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(p->d_tiles, kept.data(), kept.size() * sizeof(int64_t),
                                  cudaMemcpyHostToDevice, ctx->stream));
    // edge tiles leave part of their slot unwritten: define it
    GB_CHECK_CUDA(cudaMemsetAsync(p->d_data, 0, p->bytes, ctx->stream));
    tile_copy_kernel<<<(unsigned)p->nkept, dim3(64, 4), 0, ctx->stream>>>(
        (unsigned long long*)t->data, (unsigned long long*)p->d_data, p->d_tiles, rows, cols,
        ntr, words, 0);
    GB_CHECK_CUDA(cudaGetLastError());
    count_launch(ctx);
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // `kept` ends with this scope
  } catch (...) {
    if (p->d_tiles) cudaFreeAsync(p->d_tiles, ctx->stream);
    if (p->d_data) cudaFreeAsync(p->d_data, ctx->stream);
    delete p;
    throw;
  }
  return p;
}

void packed_unpack(gb_ctx* ctx, const gb_packed* p, gb_tensor* out) {
  GB_REQUIRE(out->kind == p->kind && out->dtype == p->dtype && out->ndim == p->ndim,
             "unpack: output kind or dtype differs from the packed tensor");
  for (int i = 0; i < p->ndim; ++i)
    GB_REQUIRE(out->dims[i] == p->dims[i], "unpack: output shape differs from the packed tensor");
  GB_CHECK_CUDA(cudaMemsetAsync(out->data, 0, out->bytes, ctx->stream));
  if (p->nkept == 0) return;
  const int words = elem_size(p->dtype) / 8;
  const int64_t ntr = (p->rows + PT - 1) / PT;
  tile_copy_kernel<<<(unsigned)p->nkept, dim3(64, 4), 0, ctx->stream>>>(
      (unsigned long long*)out->data, (unsigned long long*)p->d_data, p->d_tiles, p->rows,
      p->cols, ntr, words, 1);
  GB_CHECK_CUDA(cudaGetLastError());
  count_launch(ctx);
}

void packed_info(const gb_packed* p, int64_t* kept, int64_t* total, size_t* bytes) {
  const int64_t ntr = (p->rows + PT - 1) / PT, ntc = (p->cols + PT - 1) / PT;
  if (kept) *kept = p->nkept;
  if (total) *total = ntr * ntc;
  if (bytes) *bytes = p->bytes;
}

gb_ctx* packed_ctx(const gb_packed* p) { return p->ctx; }

void packed_free(gb_packed* p) {
  if (!p) return;
  if (p->d_tiles) cudaFreeAsync(p->d_tiles, p->ctx->stream);
  if (p->d_data) cudaFreeAsync(p->d_data, p->ctx->stream);
  delete p;
}
}  // namespace gb

