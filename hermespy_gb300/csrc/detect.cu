// Channel estimation (LS), per-element equalization (ZF / LMMSE) and the fused
// receivers that end in bit-error counts.
#include <algorithm>

#include "fading_dev.cuh"
#include "lmmse_dev.cuh"
#include "equalize_dev.cuh"

struct hpx_ls {
  const hpx_frame* frame;
  int C;          // columns of the estimate
  int ntx = 1;    // streams: one interpolation table of W*C rows each
  int nnz;
  int32_t* d_indptr = nullptr;   // [W*C + 1]
  int32_t* d_indices = nullptr;  // [nnz] reference index
  float* d_weights = nullptr;    // [nnz]
  int32_t* d_ref_word = nullptr;    // [num_refs]
  int32_t* d_ref_column = nullptr;  // [num_refs]
  int32_t* d_pos = nullptr;         // [nnz] word << 16 | column of the entry's reference element
  float2* d_coef = nullptr;         // [nnz] weight * conj(x_ref) / |x_ref|^2 (the LS division folded in)
  // staged form (k_ls_staged): per block of LS_BLOCK_ROWS rows the distinct reference
  // positions its entries read (d_bpos[d_bstart[b] .. d_bstart[b + 1])), and per entry the
  // index of its position in that list; empty if a block's list is too long to stage
  int32_t* d_bstart = nullptr;      // [blocks + 1]
  int32_t* d_bpos = nullptr;        // [sum of the lists] word << 16 | column
  int32_t* d_loc = nullptr;         // [nnz]
  int max_block_refs = 0;
};

// True if the LS table's grid (words x columns) is the frame's: the receivers lay
// the received grid out by the table's frame and columns.
bool hpx_ls_matches_frame(const hpx_ls* ls, const hpx_frame* frame) {
  const hpx_frame_info& a = ls->frame->info;
  const hpx_frame_info& b = frame->info;
  return ls->C == b.num_columns && a.num_words == b.num_words && a.num_columns == b.num_columns &&
         a.num_subcarriers == b.num_subcarriers && a.num_refs == b.num_refs;
}

namespace {

template <int NRX, int NTX>
__global__ void k_equalize(int mode, int64_t K, const float2* __restrict__ Hg, const float2* __restrict__ Yg,
                           const float* __restrict__ nv, float2* __restrict__ Xg, int out_streams) {
  const int b = blockIdx.y;
  const float s2 = nv ? nv[b] : 0.0f;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < K; k += (int64_t)gridDim.x * blockDim.x) {
    float2 H[NRX][NTX], y[NRX], x[NTX];
#pragma unroll
    for (int r = 0; r < NRX; ++r) {
      y[r] = Yg[((int64_t)b * NRX + r) * K + k];
#pragma unroll
      for (int t = 0; t < NTX; ++t) H[r][t] = Hg[(((int64_t)b * NRX + r) * NTX + t) * K + k];
    }
    equalize_one<NRX, NTX>(mode, H, y, s2, x);  // equalized symbols out: NaN inputs stay visible as NaN
    for (int t = 0; t < out_streams; ++t) Xg[((int64_t)b * out_streams + t) * K + k] = x[t];
  }
}

// Stage the packed Philox bits of data elements [k0, k0 + nd) of `nstreams`
// streams in shared memory; returns the word offset to index with absolute
// stream bit positions (words(s)[pos >> 5]).
__device__ __forceinline__ void stage_bits(uint32_t* bitsm, int BW, int nstreams, uint64_t seed, int64_t drop, int64_t k0,
                                           int nd, int m) {
  if (nd <= 0) return;
  const int64_t blk0 = ((k0 * m) >> 5) >> 2, blk1 = (((k0 + nd) * m - 1) >> 5) >> 2;
  const int nblk = (int)(blk1 - blk0 + 1);
  for (int q = threadIdx.x; q < nblk * nstreams; q += blockDim.x) {
    const int s = q / nblk;
    const int64_t blk = blk0 + (q - s * nblk);
    const uint4 r = hpx_random_block(seed, drop, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
    uint32_t* dst = bitsm + s * BW + (blk - blk0) * 4;
    dst[0] = r.x;
    dst[1] = r.y;
    dst[2] = r.z;
    dst[3] = r.w;
  }
}

// Block sum of the threads' error counts into *out; `bad` (any thread) adds the
// HPX_DROP_NUMERIC flag to the drop's word.
__device__ __forceinline__ void block_count(unsigned int local, bool bad, uint32_t* out) {
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  __shared__ unsigned int warp_sums[32];
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = local;
  const int any_bad = __syncthreads_or(bad);
  if (threadIdx.x < 32) {
    unsigned int v = threadIdx.x < (blockDim.x >> 5) ? warp_sums[threadIdx.x] : 0u;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atomicAdd(out, v);
    if (threadIdx.x == 0 && any_bad) atomicOr(out, HPX_DROP_NUMERIC);
  }
}

// Fused receivers run one block per (word, drop) whose threads stride over the
// word's data elements. The block size is picked per frame so that the strides
// cover the most data elements of a word with little idle tail, up to a cap that
// keeps the large MIMO instantiations within the register file.
constexpr int DTHREADS = 384;
template <int NRX, int NTX>
constexpr int detect_max_threads() { return NRX * NTX >= 32 ? 128 : DTHREADS; }

int detect_threads(int max_nd, int cap) {
  const int iters = max_nd > cap ? (max_nd + cap - 1) / cap : 1;
  int t = (max_nd + iters - 1) / iters;
  t = (t + 31) / 32 * 32;
  return t < 32 ? 32 : (t > cap ? cap : t);
}

// Fused ideal-CSI receiver, one block per (word, drop).
template <int NRX, int NTX>
__global__ void __launch_bounds__(detect_max_threads<NRX, NTX>()) k_detect_ideal(FadingConst fc, FadingView v, int N, int W, int C, int m,
                                                           const int32_t* __restrict__ window_start,
                                                           const int32_t* __restrict__ data_offset,
                                                           const int32_t* __restrict__ num_data_word,
                                                           const int32_t* __restrict__ data_column,
                                                           const int32_t* __restrict__ bins,
                                                           const float2* __restrict__ tw, const __grid_constant__ QamDemapTable qt, int mode,
                                                           const float2* __restrict__ grid, int gcols,
                                                           const float* __restrict__ nv, uint64_t seed, int64_t drop0,
                                                           uint32_t* __restrict__ errors) {
  extern __shared__ float4 smem4[];
  const int w = blockIdx.x, b = blockIdx.y;
  const int BW = staged_bit_words(C, m);
  float2* hb = reinterpret_cast<float2*>(smem4);
  float2* scratch = hb + fc.L;
  float2* Sm = scratch + fc.L * fc.S1;
  float2* Mg = Sm + NRX * NTX;  // S^H S
  int* ds = reinterpret_cast<int*>(Mg + NTX * NTX);
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(ds + fc.L + 4);
  const int64_t k0 = data_offset[w];
  const int nd = num_data_word[w];
  for (int l = threadIdx.x; l < fc.L; l += blockDim.x) ds[l] = fc.delay[l];
  const float2* Sg = v.spatial(b);
  for (int i = threadIdx.x; i < NRX * NTX; i += blockDim.x) Sm[i] = Sg[i];
  for (int q = threadIdx.x; q < NTX * NTX; q += blockDim.x) {
    const int i = q / NTX, j = q - i * NTX;
    float2 acc = make_float2(0.f, 0.f);
    for (int r = 0; r < NRX; ++r) cfmac(acc, Sg[r * NTX + i], Sg[r * NTX + j]);
    Mg[q] = acc;
  }
  stage_bits(bitsm, BW, NTX, seed, drop0 + b, k0, nd, m);
  tap_averages(fc, v.W(b), v.P0(b), window_start[w], N, hb, scratch);  // ends with __syncthreads
  const int64_t wofs = (((k0 * m) >> 5) >> 2) * 4;
  const float s2 = nv ? nv[b] : 0.0f;
  const int out_streams = (mode == HPX_EQ_ZF && NRX == 1) ? 1 : NTX;
  unsigned int local = 0;
  bool fin = finite_f(s2);  // a NaN / inf noise power is an invalid drop too
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    const int64_t k = k0 + j;
    const int c = data_column[k];
    const float2 g = tap_response(fc, hb, ds, tw, bins[c], N);
    float2 y[NRX], x[NTX];
#pragma unroll
    for (int r = 0; r < NRX; ++r) y[r] = grid[(((int64_t)b * NRX + r) * W + w) * gcols + c];
    if (gram_equalizer<NRX, NTX>(mode)) {  // H = S g: the Gram from S^H S (uniform branch)
      fin &= equalize_spatial<NRX, NTX>(mode, Sm, Mg, g, y, s2, x);
    } else {
      float2 H[NRX][NTX];
#pragma unroll
      for (int r = 0; r < NRX; ++r)
#pragma unroll
        for (int t = 0; t < NTX; ++t) H[r][t] = cmul(Sm[r * NTX + t], g);  // the ideal CSI of hpx_fading_ideal_csi
      fin &= equalize_one<NRX, NTX>(mode, H, y, s2, x);
    }
    // streams the equalizer does not return are received as zero bits
    // (BitErrorEvaluator zero-pads the shorter sequence)
    uint32_t dec[NTX];
    qam_decide_n<NTX>(qt, x, out_streams, dec);
#pragma unroll
    for (int t = 0; t < NTX; ++t) {
      const uint32_t rx_v = dec[t];
      const uint32_t tx_v = extract_bits_msb(bitsm + t * BW - wofs, k * m, m);
      local += __popc(rx_v ^ tx_v);
    }
  }
  block_count(local, !fin, errors + b);
}

// Fused receiver for a given CSI grid (any estimator), one block per (word, drop):
// H from csi[B][NRX][NTX][W][ccols], y from grid[B][NRX][W][gcols]. Streaming the
// channel from HBM is latency bound, so blocks stay small (at most 192 threads, each
// thread several elements) and several share an SM: the 4 x 4 kernel holds 96
// registers at 3-4 blocks per SM instead of 114 at one block of 320 threads (up to 4
// transmit streams and 16 antenna pairs; larger systems keep the wide blocks).
template <int NRX, int NTX>
constexpr bool csi_small() { return NTX <= 4 && NRX * NTX <= 16; }
template <int NRX, int NTX>
constexpr int csi_max_threads() { return csi_small<NRX, NTX>() ? 192 : detect_max_threads<NRX, NTX>(); }

template <int NRX, int NTX>
__global__ void __launch_bounds__(csi_max_threads<NRX, NTX>(), csi_small<NRX, NTX>() ? 3 : 1) k_detect_csi(
    int W, int C, int m, const int32_t* __restrict__ data_offset, const int32_t* __restrict__ num_data_word,
    const int32_t* __restrict__ data_column, const __grid_constant__ QamDemapTable qt, int mode,
    const float2* __restrict__ grid, int gcols, const float2* __restrict__ csi, int ccols,
    const float* __restrict__ nv, uint64_t seed, int64_t drop0, uint32_t* __restrict__ errors) {
  extern __shared__ float4 smem4[];
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(smem4);
  const int w = blockIdx.x, b = blockIdx.y;
  const int BW = staged_bit_words(C, m);
  const int64_t k0 = data_offset[w];
  const int nd = num_data_word[w];
  stage_bits(bitsm, BW, NTX, seed, drop0 + b, k0, nd, m);
  __syncthreads();
  const int64_t wofs = (((k0 * m) >> 5) >> 2) * 4;
  const float s2 = nv ? nv[b] : 0.0f;
  const int out_streams = (mode == HPX_EQ_ZF && NRX == 1) ? 1 : NTX;
  const int64_t hplane = (int64_t)W * ccols;  // one (rx, tx) pair of the CSI grid
  const float2* hb = csi + (int64_t)b * NRX * NTX * hplane + (int64_t)w * ccols;
  const float2* yb = grid + (int64_t)b * NRX * W * gcols + (int64_t)w * gcols;
  unsigned int local = 0;
  bool fin = finite_f(s2);  // a NaN / inf noise power is an invalid drop too
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    const int64_t k = k0 + j;
    const int c = data_column[k];
    float2 H[NRX][NTX], y[NRX], x[NTX];
#pragma unroll
    for (int r = 0; r < NRX; ++r) {
      y[r] = yb[(int64_t)r * W * gcols + c];
#pragma unroll
      for (int t = 0; t < NTX; ++t) H[r][t] = hb[(int64_t)(r * NTX + t) * hplane + c];
    }
    fin &= equalize_one<NRX, NTX>(mode, H, y, s2, x);
#pragma unroll
    for (int t = 0; t < NTX; ++t) {  // decided stream by stream: qam_decide_n spills in this kernel
      const uint32_t rx_v = t < out_streams ? qam_decide(qt, x[t]) : 0u;
      const uint32_t tx_v = extract_bits_msb(bitsm + t * BW - wofs, k * m, m);
      local += __popc(rx_v ^ tx_v);
    }
  }
  block_count(local, !fin, errors + b);
}

// Fused receiver with the tap-domain LMMSE channel estimate, one block per drop:
// the drop's tap gains of every pair and word are estimated into shared memory
// (lmmse_drop_taps) and every data element forms its channel from them, so the CSI
// grid never reaches HBM. Same estimate, equalizer, demap and count as
// hpx_lmmse_estimate + hpx_detect_csi.
constexpr int LMMSE_THREADS = 512;
template <int NRX, int NTX>
__global__ void __launch_bounds__(LMMSE_THREADS, 2) k_detect_lmmse(LmmseView e, int C, int m, int num_data,
                                                      const int32_t* __restrict__ data_column,
                                                      const int32_t* __restrict__ data_word,
                                                      const int32_t* __restrict__ bins, const float2* __restrict__ tw,
                                                      const __grid_constant__ QamDemapTable qt, int mode,
                                                      const float2* __restrict__ grid, int gcols,
                                                      const float* __restrict__ nv, uint64_t seed, int64_t drop0,
                                                      uint32_t* __restrict__ errors) {
  constexpr int NP = NRX * NTX;
  extern __shared__ float4 smem4[];
  const int b = blockIdx.x;
  const int W = e.W, U = e.U;
  float2* gt = reinterpret_cast<float2*>(smem4);
  float2* gls = gt + (size_t)W * U * NP;
  float* cw = reinterpret_cast<float*>(gls + NP * e.np * U);
  int* ds = reinterpret_cast<int*>(cw + (size_t)e.ntx * U * W * e.np);
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(ds + U + 4);
  const int BW = ((num_data * m) >> 5) + 9;  // staged words of one stream's whole frame
  stage_bits(bitsm, BW, NTX, seed, drop0 + b, 0, num_data, m);
  const float s2 = nv ? nv[b] : 0.0f;
  lmmse_drop_taps<NP>(e, b, NRX, grid, gcols, s2, gt, gls, cw, ds);  // ends with __syncthreads
  const int out_streams = (mode == HPX_EQ_ZF && NRX == 1) ? 1 : NTX;
  unsigned int local = 0;
  bool fin = finite_f(s2);  // a NaN / inf noise power is an invalid drop too
  for (int k = threadIdx.x; k < num_data; k += blockDim.x) {
    const int c = data_column[k], w = data_word[k];
    float2 hp[NP];
    lmmse_response<NP>(gt + (size_t)w * U * NP, ds, U, e.N, bins[c], tw, hp);
    float2 H[NRX][NTX], y[NRX], x[NTX];
#pragma unroll
    for (int r = 0; r < NRX; ++r) {
      y[r] = grid[(((int64_t)b * NRX + r) * W + w) * gcols + c];
#pragma unroll
      for (int t = 0; t < NTX; ++t) H[r][t] = hp[r * NTX + t];
    }
    fin &= equalize_one<NRX, NTX>(mode, H, y, s2, x);
    uint32_t dec[NTX];
    qam_decide_n<NTX>(qt, x, out_streams, dec);
#pragma unroll
    for (int t = 0; t < NTX; ++t) {
      const uint32_t rx_v = dec[t];
      const uint32_t tx_v = extract_bits_msb(bitsm + t * BW, (int64_t)k * m, m);
      local += __popc(rx_v ^ tx_v);
    }
  }
  block_count(local, !fin, errors + b);
}

// Fused SISO LS receiver, one block per (word, drop).
__global__ void __launch_bounds__(DTHREADS) k_detect_ls(int W, int C, int m, const int32_t* __restrict__ data_offset,
                                                        const int32_t* __restrict__ num_data_word,
                                                        const int32_t* __restrict__ data_column,
                                                        const int32_t* __restrict__ indptr,
                                                        const int32_t* __restrict__ indices,
                                                        const float* __restrict__ weights,
                                                        const int32_t* __restrict__ ref_word,
                                                        const int32_t* __restrict__ ref_column,
                                                        const float2* __restrict__ pilots, const __grid_constant__ QamDemapTable qt, int mode,
                                                        const float2* __restrict__ grid, int gcols,
                                                        const float* __restrict__ nv, uint64_t seed, int64_t drop0,
                                                        uint32_t* __restrict__ errors) {
  extern __shared__ float4 smem4[];
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(smem4);
  const int w = blockIdx.x, b = blockIdx.y;
  const int BW = staged_bit_words(C, m);
  const int64_t k0 = data_offset[w];
  const int nd = num_data_word[w];
  stage_bits(bitsm, BW, 1, seed, drop0 + b, k0, nd, m);
  __syncthreads();
  const int64_t wofs = (((k0 * m) >> 5) >> 2) * 4;
  const float s2 = nv ? nv[b] : 0.0f;
  const float2* gb = grid + (int64_t)b * W * gcols;
  unsigned int local = 0;
  bool fin = finite_f(s2);  // a NaN / inf noise power is an invalid drop too
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    const int64_t k = k0 + j;
    const int c = data_column[k];
    const int row = w * C + c;
    float2 h = make_float2(0.f, 0.f);
    for (int e = indptr[row]; e < indptr[row + 1]; ++e) {
      const int p = indices[e];
      const float2 yp = gb[ref_word[p] * gcols + ref_column[p]];
      const float2 xp = pilots[p];
      const float den = xp.x * xp.x + xp.y * xp.y;
      const float2 ls = make_float2((yp.x * xp.x + yp.y * xp.y) / den, (yp.y * xp.x - yp.x * xp.y) / den);
      h = cadd(h, cscale(ls, weights[e]));
    }
    float2 H[1][1] = {{h}}, y[1] = {gb[w * gcols + c]}, x[1];
    fin &= equalize_one<1, 1>(mode, H, y, s2, x);
    const uint32_t rx_v = qam_decide(qt, x[0]);
    const uint32_t tx_v = extract_bits_msb(bitsm - wofs, k * m, m);
    local += __popc(rx_v ^ tx_v);
  }
  block_count(local, !fin, errors + b);
}

// Staged LS + interpolation: one block per LS_BLOCK_ROWS table rows and LS_ITEMS
// received grids (drop, rx). The block first copies, for each of its grids, the
// reference positions its rows read (one list per row block, built with the table)
// into shared memory, then every thread walks its row's entries in table order on
// those copies: the same products and sums as k_ls_estimate, with one read of each
// reference element per grid instead of one per entry (the entries gather from L2).
constexpr int LS_BLOCK_ROWS = 256;
constexpr int LS_STAGE_ITEMS = 16;
__global__ void __launch_bounds__(LS_BLOCK_ROWS) k_ls_staged(int W, int rows, int items,
                                                              const int32_t* __restrict__ indptr,
                                                              const int32_t* __restrict__ loc,
                                                              const float2* __restrict__ coef,
                                                              const int32_t* __restrict__ bstart,
                                                              const int32_t* __restrict__ bpos,
                                                              const float2* __restrict__ grid, int gcols,
                                                              float2* __restrict__ est) {
  extern __shared__ float2 stg[];  // [LS_STAGE_ITEMS][np]
  const int blk = blockIdx.x, i0 = blockIdx.y * LS_STAGE_ITEMS;
  const int n = min(LS_STAGE_ITEMS, items - i0);
  const int p0 = bstart[blk], np = bstart[blk + 1] - p0;
  for (int q = threadIdx.x; q < np * LS_STAGE_ITEMS; q += LS_BLOCK_ROWS) {
    const int i = q / np, j = q - i * np;
    const int ps = bpos[p0 + j];
    stg[q] = i < n ? grid[(int64_t)(i0 + i) * W * gcols + (int64_t)(ps >> 16) * gcols + (ps & 0xFFFF)]
                   : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int row = blk * LS_BLOCK_ROWS + threadIdx.x;
  if (row >= rows) return;
  float2 h[LS_STAGE_ITEMS];
#pragma unroll
  for (int i = 0; i < LS_STAGE_ITEMS; ++i) h[i] = make_float2(0.f, 0.f);
  for (int e = indptr[row]; e < indptr[row + 1]; ++e) {
    const int l = loc[e];
    const float2 cf = coef[e];
#pragma unroll
    for (int i = 0; i < LS_STAGE_ITEMS; ++i) cfma(h[i], cf, stg[i * np + l]);
  }
#pragma unroll
  for (int i = 0; i < LS_STAGE_ITEMS; ++i) {
    if (i >= n) break;
    est[(int64_t)(i0 + i) * rows + row] = h[i];
  }
}

// rows = streams * W * C (the stacked tables); blockIdx.y covers LS_ITEMS received
// grids (drop, rx), which share every table row a thread loads. Each table entry is
// (position, weight conj(x) / |x|^2): the LS value y / x of a reference element and
// its interpolation weight in one complex multiply-add.
constexpr int LS_ITEMS = 16;
__global__ void __launch_bounds__(256) k_ls_estimate(int W, int rows, int items, const int32_t* __restrict__ indptr,
                                                     const int32_t* __restrict__ pos, const float2* __restrict__ coef,
                                                     const float2* __restrict__ grid, int gcols,
                                                     float2* __restrict__ est) {
  const int i0 = blockIdx.y * LS_ITEMS;
  const int n = min(LS_ITEMS, items - i0);
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < rows; row += gridDim.x * blockDim.x) {
    float2 h[LS_ITEMS];
#pragma unroll
    for (int i = 0; i < LS_ITEMS; ++i) h[i] = make_float2(0.f, 0.f);
    for (int e = indptr[row]; e < indptr[row + 1]; ++e) {
      const int ps = pos[e];
      const float2 cf = coef[e];
      const int64_t at = (int64_t)(ps >> 16) * gcols + (ps & 0xFFFF);
#pragma unroll
      for (int i = 0; i < LS_ITEMS; ++i) {
        if (i >= n) break;
        cfma(h[i], cf, grid[(int64_t)(i0 + i) * W * gcols + at]);
      }
    }
#pragma unroll
    for (int i = 0; i < LS_ITEMS; ++i) {
      if (i >= n) break;
      est[(int64_t)(i0 + i) * rows + row] = h[i];
    }
  }
}

template <int NRX>
hpx_status eq_dispatch_tx(int mode, int ntx, int64_t K, int B, const float2* H, const float2* Y, const float* nv,
                          float2* X, cudaStream_t s) {
  const int out_streams = (mode == HPX_EQ_ZF && NRX == 1) ? 1 : ntx;
  int gx = (int)((K + 255) / 256);
  if (gx > 1024) gx = 1024;
  dim3 grid(gx, B);
  switch (ntx) {
    case 1: k_equalize<NRX, 1><<<grid, 256, 0, s>>>(mode, K, H, Y, nv, X, out_streams); break;
    case 2: k_equalize<NRX, 2><<<grid, 256, 0, s>>>(mode, K, H, Y, nv, X, out_streams); break;
    case 4: k_equalize<NRX, 4><<<grid, 256, 0, s>>>(mode, K, H, Y, nv, X, out_streams); break;
    case 8: k_equalize<NRX, 8><<<grid, 128, 0, s>>>(mode, K, H, Y, nv, X, out_streams); break;
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "equalize: %d transmit streams not supported (1, 2, 4, 8)", ntx);
  }
  HPX_LAUNCHED("equalize");
  return HPX_OK;
}

template <int NRX, int NTX>
hpx_status launch_detect_ideal(const hpx_fading* f, const void* state, const hpx_frame* fr, int mode,
                               const hpx_cf32* grid, int gcols, const float* nv, uint64_t seed, int64_t drop0, int B,
                               uint32_t* errors, cudaStream_t s) {
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const FadingConst fc = fading_const(f);
  const int C = fr->info.num_columns, m = fr->info.bits_per_symbol;
  const int BW = staged_bit_words(C, m);
  const size_t smem = (size_t)fc.L * sizeof(float2) * (1 + fc.S1) + (NRX + NTX) * NTX * sizeof(float2) +
                      (fc.L + 4) * sizeof(int) + (size_t)NTX * BW * 4 + 16;
  auto kern = k_detect_ideal<NRX, NTX>;
  if (smem > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid_dim(fr->info.num_words, B);
  const int threads = detect_threads(fr->max_data_word, detect_max_threads<NRX, NTX>());
  kern<<<grid_dim, threads, smem, s>>>(fc, fading_view(f, state), fr->info.num_subcarriers, fr->info.num_words, C, m,
                                        fr->d_window_start, fr->d_data_offset, fr->d_num_data_word, fr->d_data_column,
                                        fr->d_bins, fr->d_twiddle, qt, mode, reinterpret_cast<const float2*>(grid),
                                        gcols, nv, seed, drop0, errors);
  HPX_LAUNCHED("detect_ideal");
  return HPX_OK;
}

template <int NRX, int NTX>
hpx_status launch_detect_csi(const hpx_frame* fr, int mode, const hpx_cf32* grid, int gcols, const hpx_cf32* csi,
                             int ccols, const float* nv, uint64_t seed, int64_t drop0, int B, uint32_t* errors,
                             cudaStream_t s) {
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const int C = fr->info.num_columns, m = fr->info.bits_per_symbol;
  const size_t smem = (size_t)NTX * staged_bit_words(C, m) * 4 + 16;
  auto kern = k_detect_csi<NRX, NTX>;
  if (smem > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid_dim(fr->info.num_words, B);
  const int threads = detect_threads(fr->max_data_word, csi_max_threads<NRX, NTX>());
  kern<<<grid_dim, threads, smem, s>>>(fr->info.num_words, C, m, fr->d_data_offset, fr->d_num_data_word,
                                       fr->d_data_column, qt, mode, reinterpret_cast<const float2*>(grid), gcols,
                                       reinterpret_cast<const float2*>(csi), ccols, nv, seed, drop0, errors);
  HPX_LAUNCHED("detect_csi");
  return HPX_OK;
}

template <int NRX>
hpx_status detect_csi_tx(int ntx, const hpx_frame* fr, int mode, const hpx_cf32* grid, int gcols,
                         const hpx_cf32* csi, int ccols, const float* nv, uint64_t seed, int64_t drop0, int B,
                         uint32_t* errors, cudaStream_t s) {
  switch (ntx) {
    case 1: return launch_detect_csi<NRX, 1>(fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 2: return launch_detect_csi<NRX, 2>(fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 4: return launch_detect_csi<NRX, 4>(fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 8: return launch_detect_csi<NRX, 8>(fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_csi: %d transmit streams not supported (1, 2, 4, 8)", ntx);
  }
}

template <int NRX>
hpx_status detect_ideal_tx(int ntx, const hpx_fading* f, const void* state, const hpx_frame* fr, int mode,
                           const hpx_cf32* grid, int gcols, const float* nv, uint64_t seed, int64_t drop0, int B,
                           uint32_t* errors, cudaStream_t s) {
  switch (ntx) {
    case 1: return launch_detect_ideal<NRX, 1>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 2: return launch_detect_ideal<NRX, 2>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 4: return launch_detect_ideal<NRX, 4>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 8: return launch_detect_ideal<NRX, 8>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect: %d transmit antennas not supported (1, 2, 4, 8)", ntx);
  }
}

// The staged kernel when the table has its block lists, else the gathering one.
hpx_status launch_ls(const hpx_ls* ls, int W, int rows, int items, const float2* grid, int gcols, float2* est,
                     cudaStream_t s) {
  if (ls->max_block_refs > 0) {
    const size_t smem = (size_t)LS_STAGE_ITEMS * ls->max_block_refs * sizeof(float2);
    if (smem > 48 * 1024)
      HPX_CUDA(cudaFuncSetAttribute(k_ls_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 g((rows + LS_BLOCK_ROWS - 1) / LS_BLOCK_ROWS, (items + LS_STAGE_ITEMS - 1) / LS_STAGE_ITEMS);
    k_ls_staged<<<g, LS_BLOCK_ROWS, smem, s>>>(W, rows, items, ls->d_indptr, ls->d_loc, ls->d_coef, ls->d_bstart,
                                               ls->d_bpos, grid, gcols, est);
  } else {
    dim3 g((rows + 255) / 256, (items + LS_ITEMS - 1) / LS_ITEMS);
    k_ls_estimate<<<g, 256, 0, s>>>(W, rows, items, ls->d_indptr, ls->d_pos, ls->d_coef, grid, gcols, est);
  }
  HPX_LAUNCHED("ls_estimate");
  return HPX_OK;
}

}  // namespace

extern "C" {

hpx_status hpx_ls_create_streams(const hpx_frame* frame, int32_t C, int32_t num_streams, const int32_t* indptr,
                                 const int32_t* indices, const float* weights, hpx_ls** out) {
  if (!frame || !out || !indptr) return hpx_fail(HPX_ERR_ARG, "ls: null argument");
  *out = nullptr;
  const int W = frame->info.num_words;
  if (C < frame->info.num_columns || C > frame->info.num_subcarriers)
    return hpx_fail(HPX_ERR_ARG, "ls: columns must cover the frame's resource columns");
  if (frame->info.num_refs < 1) return hpx_fail(HPX_ERR_ARG, "ls: frame has no reference elements");
  if (num_streams < 1 || num_streams > 64) return hpx_fail(HPX_ERR_ARG, "ls: num_streams must be in [1, 64]");
  if (W > 32767 || frame->info.num_columns > 65535)  // table positions pack word << 16 | column
    return hpx_fail(HPX_ERR_UNSUPPORTED, "ls: frames up to 32767 words of 65535 columns");
  if (num_streams > 1 && frame->pilot_comb < num_streams)
    return hpx_fail(HPX_ERR_UNSUPPORTED, "Least-Squares channel estimation of %d streams needs a pilot comb of at "
                                         "least %d (frame has %d)", num_streams, num_streams, frame->pilot_comb);
  const int rows = W * C * num_streams;
  const int nnz = indptr[rows];
  if (indptr[0] != 0 || nnz < 0) return hpx_fail(HPX_ERR_ARG, "ls: malformed table");
  for (int r = 0; r < rows; ++r)
    if (indptr[r + 1] < indptr[r]) return hpx_fail(HPX_ERR_ARG, "ls: malformed table");
  for (int e = 0; e < nnz; ++e)
    if (indices[e] < 0 || indices[e] >= frame->info.num_refs) return hpx_fail(HPX_ERR_ARG, "ls: index out of range");
  std::vector<int32_t> rw, rc;
  const int FC = frame->info.num_columns;
  for (int w = 0; w < W; ++w)
    for (int c = 0; c < FC; ++c)
      if (frame->h_kind[(size_t)w * FC + c] == HPX_RE_REFERENCE) {
        rw.push_back(w);
        rc.push_back(c);
      }
  hpx_ls* ls = new hpx_ls();
  ls->frame = frame;
  ls->C = C;
  ls->ntx = num_streams;
  ls->nnz = nnz;
  auto up = [](void** dst, const void* src, size_t bytes) -> cudaError_t {
    if (bytes == 0) {
      *dst = nullptr;
      return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(dst, bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  };
  cudaError_t e;
  std::vector<float2> pilots(frame->info.num_refs);
  if ((e = cudaMemcpy(pilots.data(), frame->d_pilots, pilots.size() * sizeof(float2), cudaMemcpyDeviceToHost)) !=
      cudaSuccess) {
    hpx_ls_destroy(ls);
    return hpx_cuda_status(e, "ls pilots");
  }
  std::vector<int32_t> pos(nnz);
  std::vector<float2> coef(nnz);
  for (int q = 0; q < nnz; ++q) {
    const int p = indices[q];
    const double xr = pilots[p].x, xi = pilots[p].y, den = xr * xr + xi * xi;
    pos[q] = (rw[p] << 16) | rc[p];
    coef[q] = den > 0 ? make_float2((float)(weights[q] * xr / den), (float)(-weights[q] * xi / den))
                      : make_float2(NAN, NAN);  // y / 0, as the division it replaces
  }
  // staged form: the distinct positions read by each block of LS_BLOCK_ROWS rows
  const int nblk = (rows + LS_BLOCK_ROWS - 1) / LS_BLOCK_ROWS;
  std::vector<int32_t> bstart(nblk + 1, 0), bpos, loc(nnz);
  for (int b = 0; b < nblk; ++b) {
    const int e0 = indptr[b * LS_BLOCK_ROWS], e1 = indptr[std::min(rows, (b + 1) * LS_BLOCK_ROWS)];
    std::vector<int32_t> u(pos.begin() + e0, pos.begin() + e1);
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    for (int q = e0; q < e1; ++q) loc[q] = (int32_t)(std::lower_bound(u.begin(), u.end(), pos[q]) - u.begin());
    bstart[b] = (int32_t)bpos.size();
    bpos.insert(bpos.end(), u.begin(), u.end());
    ls->max_block_refs = std::max(ls->max_block_refs, (int)u.size());
  }
  bstart[nblk] = (int32_t)bpos.size();
  const bool staged = (size_t)LS_STAGE_ITEMS * ls->max_block_refs * sizeof(float2) <= 96 * 1024 && nnz > 0;
  if (!staged) ls->max_block_refs = 0;
  if ((e = up((void**)&ls->d_indptr, indptr, (rows + 1) * sizeof(int32_t))) != cudaSuccess ||
      (staged && (e = up((void**)&ls->d_bstart, bstart.data(), bstart.size() * sizeof(int32_t))) != cudaSuccess) ||
      (staged && (e = up((void**)&ls->d_bpos, bpos.data(), bpos.size() * sizeof(int32_t))) != cudaSuccess) ||
      (staged && (e = up((void**)&ls->d_loc, loc.data(), loc.size() * sizeof(int32_t))) != cudaSuccess) ||
      (e = up((void**)&ls->d_indices, indices, nnz * sizeof(int32_t))) != cudaSuccess ||
      (e = up((void**)&ls->d_weights, weights, nnz * sizeof(float))) != cudaSuccess ||
      (e = up((void**)&ls->d_ref_word, rw.data(), rw.size() * sizeof(int32_t))) != cudaSuccess ||
      (e = up((void**)&ls->d_ref_column, rc.data(), rc.size() * sizeof(int32_t))) != cudaSuccess ||
      (e = up((void**)&ls->d_pos, pos.data(), nnz * sizeof(int32_t))) != cudaSuccess ||
      (e = up((void**)&ls->d_coef, coef.data(), nnz * sizeof(float2))) != cudaSuccess) {
    hpx_ls_destroy(ls);
    return hpx_cuda_status(e, "ls tables");
  }
  *out = ls;
  return HPX_OK;
}

hpx_status hpx_ls_create(const hpx_frame* frame, int32_t C, const int32_t* indptr, const int32_t* indices,
                         const float* weights, hpx_ls** out) {
  return hpx_ls_create_streams(frame, C, 1, indptr, indices, weights, out);
}

hpx_status hpx_ls_destroy(hpx_ls* ls) {
  if (!ls) return HPX_OK;
  void* p[] = {ls->d_indptr, ls->d_indices, ls->d_weights, ls->d_ref_word, ls->d_ref_column, ls->d_pos, ls->d_coef,
               ls->d_bstart, ls->d_bpos, ls->d_loc};
  for (void* q : p)
    if (q) cudaFree(q);
  delete ls;
  return HPX_OK;
}

hpx_status hpx_ls_estimate(const hpx_ls* ls, const hpx_cf32* grid, int32_t gcols, int32_t B, hpx_cf32* est,
                           void* stream) {
  if (!ls || !grid || !est) return hpx_fail(HPX_ERR_ARG, "ls_estimate: null argument");
  if (B < 0) return hpx_fail(HPX_ERR_ARG, "ls_estimate: negative batch");
  if (gcols < ls->frame->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "ls_estimate: grid too narrow");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "ls_estimate: batch too large");
  if (ls->ntx != 1) return hpx_fail(HPX_ERR_ARG, "ls_estimate: table of %d streams (use hpx_ls_estimate_streams)", ls->ntx);
  const int W = ls->frame->info.num_words;
  return launch_ls(ls, W, W * ls->C, B, reinterpret_cast<const float2*>(grid), gcols, reinterpret_cast<float2*>(est),
                   as_stream(stream));
}

hpx_status hpx_ls_estimate_streams(const hpx_ls* ls, const hpx_cf32* grid, int32_t gcols, int32_t nrx, int32_t B,
                                   hpx_cf32* est, void* stream) {
  if (!ls || !grid || !est) return hpx_fail(HPX_ERR_ARG, "ls_estimate: null argument");
  if (B < 0 || nrx < 1) return hpx_fail(HPX_ERR_ARG, "ls_estimate: bad batch");
  if (gcols < ls->frame->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "ls_estimate: grid too narrow");
  if (B == 0) return HPX_OK;
  if ((int64_t)B * nrx > 65535) return hpx_fail(HPX_ERR_ARG, "ls_estimate: batch too large");
  const int W = ls->frame->info.num_words;
  const int rows = ls->ntx * W * ls->C;
  return launch_ls(ls, W, rows, B * nrx, reinterpret_cast<const float2*>(grid), gcols, reinterpret_cast<float2*>(est),
                   as_stream(stream));
}

hpx_status hpx_equalize(int32_t mode, int32_t nrx, int32_t ntx, int64_t K, int32_t B, const hpx_cf32* H,
                        const hpx_cf32* Y, const float* nv, hpx_cf32* X, void* stream) {
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "equalize: unknown mode %d", mode);
  if (K < 0 || B < 0) return hpx_fail(HPX_ERR_ARG, "equalize: negative size");
  if (K == 0 || B == 0) return HPX_OK;
  if (!H || !Y || !X) return hpx_fail(HPX_ERR_ARG, "equalize: null buffer");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "equalize: LMMSE needs noise variances");
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "equalize: batch too large");
  const float2* h = reinterpret_cast<const float2*>(H);
  const float2* y = reinterpret_cast<const float2*>(Y);
  float2* x = reinterpret_cast<float2*>(X);
  cudaStream_t s = as_stream(stream);
  switch (nrx) {
    case 1: return eq_dispatch_tx<1>(mode, ntx, K, B, h, y, nv, x, s);
    case 2: return eq_dispatch_tx<2>(mode, ntx, K, B, h, y, nv, x, s);
    case 4: return eq_dispatch_tx<4>(mode, ntx, K, B, h, y, nv, x, s);
    case 8: return eq_dispatch_tx<8>(mode, ntx, K, B, h, y, nv, x, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "equalize: %d receive streams not supported (1, 2, 4, 8)", nrx);
  }
}

hpx_status hpx_detect_ideal(const hpx_fading* f, const void* state, const hpx_frame* fr, int32_t mode,
                            const hpx_cf32* grid, int32_t gcols, const float* nv, uint64_t seed, int64_t drop0,
                            int32_t B, uint32_t* errors, void* stream) {
  if (!f || !state || !fr || !grid || !errors) return hpx_fail(HPX_ERR_ARG, "detect_ideal: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_ideal: unknown mode");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "detect_ideal: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_ideal: bad drop range");
  if (gcols < fr->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "detect_ideal: grid too narrow");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_ideal: batch above 65535 drops per call");
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  switch (f->nrx) {
    case 1: return detect_ideal_tx<1>(f->ntx, f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 2: return detect_ideal_tx<2>(f->ntx, f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 4: return detect_ideal_tx<4>(f->ntx, f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    case 8: return detect_ideal_tx<8>(f->ntx, f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_ideal: %d receive antennas not supported", f->nrx);
  }
}

hpx_status hpx_detect_csi(const hpx_frame* fr, int32_t nrx, int32_t ntx, int32_t mode, const hpx_cf32* grid,
                          int32_t gcols, const hpx_cf32* csi, int32_t ccols, const float* nv, uint64_t seed,
                          int64_t drop0, int32_t B, uint32_t* errors, void* stream) {
  if (!fr || !grid || !csi || !errors) return hpx_fail(HPX_ERR_ARG, "detect_csi: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_csi: unknown mode");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "detect_csi: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_csi: bad drop range");
  if (gcols < fr->info.num_columns || ccols < fr->info.num_columns)
    return hpx_fail(HPX_ERR_SHAPE, "detect_csi: grid or CSI narrower than the frame");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_csi: batch above 65535 drops per call");
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  switch (nrx) {
    case 1: return detect_csi_tx<1>(ntx, fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 2: return detect_csi_tx<2>(ntx, fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 4: return detect_csi_tx<4>(ntx, fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    case 8: return detect_csi_tx<8>(ntx, fr, mode, grid, gcols, csi, ccols, nv, seed, drop0, B, errors, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_csi: %d receive streams not supported (1, 2, 4, 8)", nrx);
  }
}

hpx_status hpx_detect_lmmse(const hpx_lmmse* lm, int32_t nrx, int32_t mode, const hpx_cf32* grid, int32_t gcols,
                            const float* nv, uint64_t seed, int64_t drop0, int32_t B, uint32_t* errors,
                            void* stream) {
  if (!lm || !grid || !errors) return hpx_fail(HPX_ERR_ARG, "detect_lmmse: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_lmmse: unknown mode");
  if ((mode == HPX_EQ_LMMSE) && !nv) return hpx_fail(HPX_ERR_ARG, "detect_lmmse: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_lmmse: bad drop range");
  const hpx_frame* fr = lm->frame;
  if (gcols < fr->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "detect_lmmse: grid too narrow");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_lmmse: batch above 65535 drops per call");
  const int ntx = lm->ntx, m = fr->info.bits_per_symbol, nd = fr->info.num_data;
  if (!((nrx == 1 && ntx == 1) || (nrx == 2 && ntx == 2) || (nrx == 4 && ntx == 4) || (nrx == 4 && ntx == 2) ||
        (nrx == 2 && ntx == 1) || (nrx == 4 && ntx == 1)))
    return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_lmmse: %dx%d antennas not supported", nrx, ntx);
  // tensor-core response GEMM (lmmse_tc.cu). Its batched pilot LS stages at most 8 pilots
  // of a stream per 32 columns under the comb of 4 that 4 streams need; a layout whose
  // staging would not fit shared memory takes the FP32 kernel below instead.
  if (nrx == 4 && ntx == 4 && lm->d_tc_ftab && lm->tc_ls_stages > 0) {
    cudaStream_t s = as_stream(stream);
    HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
    return lmmse_tc_detect(lm, mode, reinterpret_cast<const float2*>(grid), gcols, nv, seed, drop0, B, errors, s);
  }
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const size_t smem = lmmse_taps_smem(lm->W, lm->U, lm->np, ntx, nrx * ntx) + 16 +
                      (size_t)ntx * ((((size_t)nd * m) >> 5) + 9) * 4;
  if (smem > 220 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_lmmse: frame needs %zu bytes of shared memory", smem);
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  const LmmseView v = lmmse_view(lm);
  auto launch = [&](auto kern) -> hpx_status {
    HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<B, LMMSE_THREADS, smem, s>>>(v, fr->info.num_columns, m, nd, fr->d_data_column, fr->d_data_word, fr->d_bins,
                              fr->d_twiddle, qt, mode, reinterpret_cast<const float2*>(grid), gcols, nv, seed, drop0,
                              errors);
    HPX_LAUNCHED("detect_lmmse");
    return HPX_OK;
  };
  if (nrx == 1) return ntx == 1 ? launch(k_detect_lmmse<1, 1>) : hpx_fail(HPX_ERR_UNSUPPORTED, "detect_lmmse");
  if (nrx == 2) return ntx == 1 ? launch(k_detect_lmmse<2, 1>) : launch(k_detect_lmmse<2, 2>);
  if (ntx == 1) return launch(k_detect_lmmse<4, 1>);
  if (ntx == 2) return launch(k_detect_lmmse<4, 2>);
  return launch(k_detect_lmmse<4, 4>);
}

// Sticky status word of the tensor-core receiver (d_tc_fail): 1 after a bounded
// wait ran out. Handles without the tensor-core path have no word and report OK.
hpx_status hpx_lmmse_status(hpx_lmmse* lm, int32_t clear, void* stream) {
  if (!lm) return hpx_fail(HPX_ERR_ARG, "lmmse_status: null argument");
  if (!lm->d_tc_fail) return HPX_OK;
  cudaStream_t s = as_stream(stream);
  int flag = 0;
  HPX_CUDA(cudaMemcpyAsync(&flag, lm->d_tc_fail, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (clear) HPX_CUDA(cudaMemsetAsync(lm->d_tc_fail, 0, sizeof(int), s));
  HPX_CUDA(cudaStreamSynchronize(s));
  if (flag) return hpx_fail(HPX_ERR_TIMEOUT, "detect_lmmse: a bounded tensor-core wait ran out (drops flagged)");
  return HPX_OK;
}

hpx_status hpx_lmmse_inject_timeout(hpx_lmmse* lm, void* stream) {
  if (!lm) return hpx_fail(HPX_ERR_ARG, "lmmse_inject_timeout: null argument");
  if (!lm->d_tc_fail) return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse_inject_timeout: the handle has no tensor-core path");
  HPX_CUDA(cudaMemsetAsync(lm->d_tc_fail, 0x01, 1, as_stream(stream)));  // the int word becomes 1
  return HPX_OK;
}

hpx_status hpx_detect_ls(const hpx_ls* ls, int32_t mode, const hpx_cf32* grid, int32_t gcols, const float* nv,
                         uint64_t seed, int64_t drop0, int32_t B, uint32_t* errors, void* stream) {
  if (!ls || !grid || !errors) return hpx_fail(HPX_ERR_ARG, "detect_ls: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_ls: unknown mode");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "detect_ls: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_ls: bad drop range");
  const hpx_frame* fr = ls->frame;
  if (ls->ntx != 1) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_ls: SISO tables only (use hpx_detect_csi)");
  if (gcols < fr->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "detect_ls: grid too narrow");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_ls: batch above 65535 drops per call");
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  const int C = ls->C, m = fr->info.bits_per_symbol;
  const size_t smem = (size_t)staged_bit_words(C, m) * 4 + 16;
  dim3 grid_dim(fr->info.num_words, B);
  k_detect_ls<<<grid_dim, detect_threads(fr->max_data_word, DTHREADS), smem, s>>>(fr->info.num_words, C, m, fr->d_data_offset, fr->d_num_data_word,
                                               fr->d_data_column, ls->d_indptr, ls->d_indices, ls->d_weights,
                                               ls->d_ref_word, ls->d_ref_column, fr->d_pilots, qt, mode,
                                               reinterpret_cast<const float2*>(grid), gcols, nv, seed, drop0, errors);
  HPX_LAUNCHED("detect_ls");
  return HPX_OK;
}

}  // extern "C"
