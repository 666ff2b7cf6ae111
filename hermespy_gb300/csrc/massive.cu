// Massive-MIMO receiver: per-element Gram and matched filter on the BF16 tensor
// cores with split (3-term) products, FP32 Cholesky LMMSE / ZF, FP64 only for the
// elements whose Cholesky condition estimate exceeds 1e6, exact hard demap and
// bit-error count. No counterpart in the reference (its MIMO equalizer is a
// per-element numpy pinv, modem/waveform.py:235-250, limited to small arrays).
//
// Per resource element with H (NRX x 16) and y (NRX):
//   P = [Re H; Im H] (2 NRX x 16), Q = [Im H; -Re H], Y = [[Re y, Im y]; [Im y, -Re y]]
//   Re(H^H H) = P^T P,  Im(H^H H) = P^T Q,  H^H y = P^T Y   (K = 2 NRX real GEMMs)
// Every operand is split X = X_hi + X_lo into two BF16 numbers and each Gram product
// is X_hi Y_hi + X_hi Y_lo + X_lo Y_hi with FP32 accumulation (mma.sync m16n8k16): the
// dropped X_lo Y_lo term is below 2^-16 of the product. The matched filter keeps all
// four terms: Y_hi and Y_lo sit side by side in one 8-column B tile, so two MMAs per
// k-step give them.
// The warp computes the Gram of two elements, then each half-warp factors one of
// them with its 16 rows in registers (lane i holds row i; packed FP32x2 updates),
// solves (forward substitution on rows, backward on columns after a transpose through
// shared memory), demaps its 16 streams and counts errors against the Philox bits,
// regenerated per element.
// The split operands are built per element from the channel h = g S (tap response g
// of the element, spatial matrix S of the drop): each lane forms 8 columns of one row,
// converts them two at a time (BF16x2 and its residual) and writes 16-byte chunks.
#include <cuda_bf16.h>

#include "fading_dev.cuh"

namespace {

constexpr int MT = 16;       // transmit streams (users)
constexpr int MWARPS = 4;
constexpr float kCondLimit = 1e6f;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// 3-term split product accumulate: c += Ahi Bhi + Ahi Blo + Alo Bhi
__device__ __forceinline__ void mma3(float (&c)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4], uint32_t bh0,
                                     uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  mma16816(c, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  mma16816(c, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  mma16816(c, al[0], al[1], al[2], al[3], bh0, bh1);
}

__device__ __forceinline__ uint32_t neg2(uint32_t v) { return v ^ 0x80008000u; }

// Byte offset of element (row, col) of a [rows][16] bf16 tile whose two 16-byte
// halves swap on every other group of 4 rows (conflict-free 8-row ldmatrix).
__device__ __forceinline__ int toff(int row, int col) {
  return row * 32 + ((((col >> 3) ^ (row >> 2)) & 1) << 4) + (col & 7) * 2;
}

// Serial FP64 Cholesky solve of (G + reg I) x = b for one element whose FP32
// factorization was ill-conditioned; G (lower triangle, overwritten by L) and b
// were formed in FP64 from the element's channel.
__device__ bool solve_fp64(double2* L, const double2* b, double reg, float2* x) {
  for (int i = 0; i < MT; ++i) {
    L[i * MT + i].x += reg;
    L[i * MT + i].y = 0.0;
  }
  for (int k = 0; k < MT; ++k) {
    double d = L[k * MT + k].x;
    for (int p = 0; p < k; ++p) d -= L[k * MT + p].x * L[k * MT + p].x + L[k * MT + p].y * L[k * MT + p].y;
    if (!(d > 0.0)) return false;
    const double pk = sqrt(d);
    L[k * MT + k] = make_double2(pk, 0.0);
    for (int i = k + 1; i < MT; ++i) {
      double2 s = L[i * MT + k];
      for (int p = 0; p < k; ++p) {
        const double2 a = L[i * MT + p], c = L[k * MT + p];  // s -= a conj(c)
        s.x -= a.x * c.x + a.y * c.y;
        s.y -= a.y * c.x - a.x * c.y;
      }
      L[i * MT + k] = make_double2(s.x / pk, s.y / pk);
    }
  }
  double2 z[MT];
  for (int i = 0; i < MT; ++i) {
    double2 s = b[i];
    for (int p = 0; p < i; ++p) {
      const double2 a = L[i * MT + p];
      s.x -= a.x * z[p].x - a.y * z[p].y;
      s.y -= a.x * z[p].y + a.y * z[p].x;
    }
    z[i] = make_double2(s.x / L[i * MT + i].x, s.y / L[i * MT + i].x);
  }
  for (int i = MT - 1; i >= 0; --i) {
    double2 s = z[i];
    for (int p = i + 1; p < MT; ++p) {
      const double2 a = L[p * MT + i];  // conj(L[p][i]) * z[p]
      s.x -= a.x * z[p].x + a.y * z[p].y;
      s.y -= a.x * z[p].y - a.y * z[p].x;
    }
    z[i] = make_double2(s.x / L[i * MT + i].x, s.y / L[i * MT + i].x);
  }
  for (int i = 0; i < MT; ++i) x[i] = make_float2((float)z[i].x, (float)z[i].y);
  return true;
}

// Stream bits of one data element, MSB first (the layout extract_bits_msb reads from
// staged words: stream bit p is bit p % 32 of word p / 32, four words per Philox
// block), generated on demand: the lane keeps the last Philox block it made, which
// serves the following elements of its stream until their bits move past it.
struct BitCache {
  int64_t blk = -1;
  uint4 cur = make_uint4(0u, 0u, 0u, 0u);
};

__device__ __forceinline__ uint32_t element_bits(BitCache& bc, uint64_t seed, int64_t drop, uint32_t stream, int64_t pos,
                                                 int m) {
  const int64_t blk = pos >> 7;
  if (blk != bc.blk) {
    bc.cur = hpx_random_block(seed, drop, stream, HPX_DOMAIN_BITS, (uint32_t)blk);
    bc.blk = blk;
  }
  const int off = (int)(pos & 127), wi = off >> 5, sh = off & 31;
  const uint32_t w0 = wi == 0 ? bc.cur.x : (wi == 1 ? bc.cur.y : (wi == 2 ? bc.cur.z : bc.cur.w));
  uint32_t w1 = wi == 0 ? bc.cur.y : (wi == 1 ? bc.cur.z : bc.cur.w);
  if (wi == 3) w1 = sh + m > 32 ? hpx_random_block(seed, drop, stream, HPX_DOMAIN_BITS, (uint32_t)(blk + 1)).x : 0u;
  const uint64_t win = (uint64_t)w0 | ((uint64_t)w1 << 32);
  const uint32_t raw = (uint32_t)(win >> sh) & ((1u << m) - 1u);
  return __brev(raw) >> (32 - m);
}

// Two floats as a BF16 pair (hi) and the pair of their rounding residuals (lo); the
// residual v - hi is exact in FP32 and formed by one packed FMA.
__device__ __forceinline__ void split2_bf16(float2 v, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __float22bfloat162_rn(v);
  const float2 r = __ffma2_rn(__bfloat1622float2(h), make_float2(-1.f, -1.f), v);
  const __nv_bfloat162 l = __float22bfloat162_rn(r);
  memcpy(&hi, &h, sizeof(hi));
  memcpy(&lo, &l, sizeof(lo));
}

// Per-warp shared memory: [P_hi | P_lo] (reused for the FP64 Gram of the two elements
// once the FP32 ones are formed), Y [KR][8] (16-byte rows: columns 0-1 hi, 2-3 lo,
// 4-7 zero), G[2][16][17] (rows padded: a half-warp reading one row per lane hits
// distinct banks; reused to transpose L), b[2][16], x[2][16] (FP64-path results),
// Cholesky column broadcast [2][16] as (re, re, im, im) (reused for the FP64 matched
// filter), g[2], column[2].
template <int NRX>
struct MassiveSmem {
  static constexpr int KR = 2 * NRX;        // stacked real rows
  static constexpr int TILE = KR * 16 * 2;  // bytes of one [KR][16] bf16 tile
  static constexpr int UNION = 2 * TILE > 2 * MT * MT * 16 ? 2 * TILE : 2 * MT * MT * 16;
  static constexpr int YBYTES = KR * 16;
  static constexpr int WARP_BYTES = UNION + YBYTES + 2 * MT * (MT + 1) * 8 + 2 * MT * 8 + 2 * MT * 8 + 2 * MT * 16 +
                                    2 * 8 + 2 * 8;
};
// Spatial matrix in shared memory as planes per row: 16 real parts, 16 imaginary parts,
// 4 floats of padding (144-byte rows: conflict-free 16-byte loads by rows)
constexpr int SMF = 2 * MT + 4;

// Fused ideal-CSI massive-MIMO receiver, one block (4 warps) per (word, drop).
template <int NRX>
__global__ void __launch_bounds__(MWARPS * 32, 3) k_detect_massive(
    FadingConst fc, FadingView v, int N, int W, int C, int m, const int32_t* __restrict__ window_start,
    const int32_t* __restrict__ data_offset, const int32_t* __restrict__ num_data_word,
    const int32_t* __restrict__ data_column, const int32_t* __restrict__ bins, const float2* __restrict__ tw,
    const __grid_constant__ QamDemapTable qt, int mode, const float2* __restrict__ grid, int gcols,
    const float* __restrict__ nv, uint64_t seed, int64_t drop0, uint32_t* __restrict__ errors,
    uint32_t* __restrict__ fp64_count, float2* __restrict__ equalized, int num_data) {
  using SM = MassiveSmem<NRX>;
  constexpr int KR = SM::KR, KS = KR / 16;
  extern __shared__ float4 smem4[];
  const int w = blockIdx.x, b = blockIdx.y;
  unsigned char* base = reinterpret_cast<unsigned char*>(smem4);
  // [NRX][SMF] spatial matrix (16-byte aligned rows), then taps
  float* Sm = reinterpret_cast<float*>(base + MWARPS * SM::WARP_BYTES);
  float2* hb = reinterpret_cast<float2*>(Sm + NRX * SMF);
  float2* scratch = hb + fc.L;
  int* ds = reinterpret_cast<int*>(scratch + fc.L * fc.S1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* my = base + warp * SM::WARP_BYTES;
  unsigned char* Phi = my;
  unsigned char* Plo = my + SM::TILE;
  unsigned char* Yt = my + SM::UNION;
  constexpr int GS = MT + 1;                                               // padded Gram row
  float2* Gs = reinterpret_cast<float2*>(Yt + SM::YBYTES);                 // [2][16][17]
  float2* bs = Gs + 2 * MT * GS;                                           // [2][16]
  float2* xs = bs + 2 * MT;                                                // [2][16] FP64-path results
  float4* colb = reinterpret_cast<float4*>(xs + 2 * MT);                   // [2][16] (re, re, im, im)
  float2* gsave = reinterpret_cast<float2*>(colb + 2 * MT);                // [2] tap response of each element
  int* csave = reinterpret_cast<int*>(gsave + 2);                          // [2] grid column of each element

  const int64_t k0 = data_offset[w];
  const int nd = num_data_word[w];
  for (int l = threadIdx.x; l < fc.L; l += blockDim.x) ds[l] = fc.delay[l];
  const float2* Sg = v.spatial(b);
  for (int i = threadIdx.x; i < NRX * MT; i += blockDim.x) {
    const float2 sv = Sg[i];
    Sm[(i / MT) * SMF + i % MT] = sv.x;
    Sm[(i / MT) * SMF + MT + i % MT] = sv.y;
  }
  // zero the Y tile once: only columns 0-3 change per element
  for (int i = lane; i < KR * 4; i += 32) reinterpret_cast<uint32_t*>(Yt)[i] = 0u;
  tap_averages(fc, v.W(b), v.P0(b), window_start[w], N, hb, scratch);  // ends with __syncthreads
  const float s2 = nv ? nv[b] : 0.0f;
  const float reg = mode == HPX_EQ_LMMSE ? s2 : 0.0f;
  const uint32_t phi = smem_u32(Phi), plo = smem_u32(Plo), yt = smem_u32(Yt);
  const int j8 = lane >> 3, r8 = lane & 7;
  const int half = lane >> 4, row = lane & 15;
  unsigned int local = 0, n64 = 0;
  BitCache bc;
  // a NaN / inf noise power, or an element whose solution (after the FP64 re-solve of
  // ill-conditioned elements) is not finite
  bool bad = !(fabsf(s2) < INFINITY);

  // received samples of the next element pair are loaded one iteration ahead
  constexpr int YR = (NRX + 31) / 32;
  float2 ypf[2][YR];
  int cpf[2];
  auto prefetch = [&](int jbase) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = jbase + s;
      cpf[s] = j < nd ? data_column[k0 + j] : 0;
#pragma unroll
      for (int q = 0; q < YR; ++q) {
        const int r = lane + 32 * q;
        ypf[s][q] = (j < nd && r < NRX) ? __ldg(grid + (((int64_t)b * NRX + r) * W + w) * gcols + cpf[s])
                                        : make_float2(0.f, 0.f);
      }
    }
  };
  prefetch(warp * 2);
  for (int j0 = warp * 2; j0 < nd; j0 += 2 * MWARPS) {
    float2 ycur[2][YR];
    int ccur[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      ccur[s] = cpf[s];
#pragma unroll
      for (int q = 0; q < YR; ++q) ycur[s][q] = ypf[s][q];
    }
    if (j0 + 2 * MWARPS < nd) prefetch(j0 + 2 * MWARPS);
    // tap responses of both elements at once: lanes 0-15 the first, 16-31 the second
    const float2 gh = tap_response(fc, hb, ds, tw, bins[half ? ccur[1] : ccur[0]], N);
    if (row == 0) {
      gsave[half] = gh;
      csave[half] = half ? ccur[1] : ccur[0];
    }
    // ---------------- Gram and matched filter of elements j0 and j0 + 1
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = j0 + s;
      float2* G = Gs + s * MT * GS;
      float2* bv = bs + s * MT;
      if (j >= nd) {  // no element: an identity system keeps the half-warp's arithmetic finite
        for (int i = lane; i < MT * MT; i += 32) G[(i / MT) * GS + i % MT] = make_float2((i % (MT + 1)) == 0 ? 1.f : 0.f, 0.f);
        if (lane < MT) bv[lane] = make_float2(0.f, 0.f);
        __syncwarp();
        continue;
      }
      const float gx = __shfl_sync(0xffffffffu, gh.x, 16 * s), gy = __shfl_sync(0xffffffffu, gh.y, 16 * s);
      const float2 gx2 = make_float2(gx, gx), gy2 = make_float2(gy, gy), ngy2 = make_float2(-gy, -gy);
      // P tiles: item = (row r, 8-column half cb); rows r (Re H) and NRX + r (Im H). Two
      // columns per packed FMA: Re h = Re s gx - Im s gy, Im h = Re s gy + Im s gx.
#pragma unroll
      for (int it = lane; it < 2 * NRX; it += 32) {
        const int r = it >> 1, cb = it & 1;
        const float4* rp = reinterpret_cast<const float4*>(Sm + r * SMF + cb * 8);
        const float4* ip = reinterpret_cast<const float4*>(Sm + r * SMF + MT + cb * 8);
        float2 hr[4], hi[4];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float4 sr = rp[q], si = ip[q];
          const float2 sr0 = make_float2(sr.x, sr.y), sr1 = make_float2(sr.z, sr.w);
          const float2 si0 = make_float2(si.x, si.y), si1 = make_float2(si.z, si.w);
          hr[2 * q] = __ffma2_rn(si0, ngy2, __fmul2_rn(sr0, gx2));
          hr[2 * q + 1] = __ffma2_rn(si1, ngy2, __fmul2_rn(sr1, gx2));
          hi[2 * q] = __ffma2_rn(si0, gx2, __fmul2_rn(sr0, gy2));
          hi[2 * q + 1] = __ffma2_rn(si1, gx2, __fmul2_rn(sr1, gy2));
        }
        uint4 rh, rl, ih, il;
        split2_bf16(hr[0], rh.x, rl.x);
        split2_bf16(hr[1], rh.y, rl.y);
        split2_bf16(hr[2], rh.z, rl.z);
        split2_bf16(hr[3], rh.w, rl.w);
        split2_bf16(hi[0], ih.x, il.x);
        split2_bf16(hi[1], ih.y, il.y);
        split2_bf16(hi[2], ih.z, il.z);
        split2_bf16(hi[3], ih.w, il.w);
        *reinterpret_cast<uint4*>(Phi + toff(r, cb * 8)) = rh;
        *reinterpret_cast<uint4*>(Plo + toff(r, cb * 8)) = rl;
        *reinterpret_cast<uint4*>(Phi + toff(NRX + r, cb * 8)) = ih;
        *reinterpret_cast<uint4*>(Plo + toff(NRX + r, cb * 8)) = il;
      }
      // Y tile: row r = [Re y, Im y], row NRX + r = [Im y, -Re y]; hi in columns 0-1, lo in 2-3
#pragma unroll
      for (int q = 0; q < YR; ++q) {
        const int r = lane + 32 * q;
        if (r >= NRX) continue;
        const float2 yv = ycur[s][q];
        uint32_t h0, l0, h1, l1;
        split2_bf16(yv, h0, l0);
        split2_bf16(make_float2(yv.y, -yv.x), h1, l1);
        *reinterpret_cast<uint2*>(Yt + r * 16) = make_uint2(h0, l0);
        *reinterpret_cast<uint2*>(Yt + (NRX + r) * 16) = make_uint2(h1, l1);
      }
      __syncwarp();
      float gr[2][4] = {}, gi[2][4] = {}, by[4] = {};
#pragma unroll
      for (int ks = 0; ks < KS / 2; ++ks) {
        const int ks2 = ks + KS / 2;
        // A = P^T fragments of k-steps ks (rows of Re H) and ks2 (rows of Im H)
        // and the same matrices in B order (a0, a2, a1, a3): the B pair of n-tile nt is
        // registers 2 nt, 2 nt + 1 of it, consecutive as the MMA wants them
        uint32_t bh[2][4], bl[2][4];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const int kk = p == 0 ? ks : ks2;
          const int rb = kk * 16 + (j8 & 1) * 8 + r8, cb2 = (j8 >> 1) * 8;
          ldsm_x4_t(phi + toff(rb, cb2), bh[p][0], bh[p][1], bh[p][2], bh[p][3]);
          ldsm_x4_t(plo + toff(rb, cb2), bl[p][0], bl[p][1], bl[p][2], bl[p][3]);
        }
        // Y fragments of both k-steps: matrices (ks, k 0-7), (ks, k 8-15), (ks2, k 0-7), (ks2, k 8-15)
        uint32_t yf[4];
        ldsm_x4_t(yt + ((j8 >> 1 ? ks2 : ks) * 16 + (j8 & 1) * 8 + r8) * 16, yf[0], yf[1], yf[2], yf[3]);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          uint32_t ah[4], al[4];  // A order, loaded per k-step to keep registers down
          {
            const int rr = (p == 0 ? ks : ks2) * 16 + (j8 >> 1) * 8 + r8, cc = (j8 & 1) * 8;
            ldsm_x4_t(phi + toff(rr, cc), ah[0], ah[1], ah[2], ah[3]);
            ldsm_x4_t(plo + toff(rr, cc), al[0], al[1], al[2], al[3]);
          }
          // B = P fragments of the same k-step (B order), Q those of the partner k-step
          const int q = 1 - p;  // Q = [Im H; -Re H]: the partner k-step, negated in the lower half
#pragma unroll
          for (int nt = 0; nt < 2; ++nt) {
            mma3(gr[nt], ah, al, bh[p][2 * nt], bh[p][2 * nt + 1], bl[p][2 * nt], bl[p][2 * nt + 1]);
            uint32_t qh0 = bh[q][2 * nt], qh1 = bh[q][2 * nt + 1], ql0 = bl[q][2 * nt], ql1 = bl[q][2 * nt + 1];
            if (p == 1) {
              qh0 = neg2(qh0);
              qh1 = neg2(qh1);
              ql0 = neg2(ql0);
              ql1 = neg2(ql1);
            }
            mma3(gi[nt], ah, al, qh0, qh1, ql0, ql1);
          }
          // matched filter: (P_hi + P_lo)^T [Y_hi | Y_lo], the lo half summed in below
          mma16816(by, ah[0], ah[1], ah[2], ah[3], yf[2 * p], yf[2 * p + 1]);
          mma16816(by, al[0], al[1], al[2], al[3], yf[2 * p], yf[2 * p + 1]);
        }
      }
      // C fragments: rows lane/4 (+8), columns 2 (lane % 4) (+1) of each 8-column tile
      const int gm = lane >> 2, gn = (lane & 3) * 2;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int hr = 0; hr < 2; ++hr)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int i = gm + hr * 8, jj = nt * 8 + gn + e;
            G[i * GS + jj] = make_float2(gr[nt][hr * 2 + e], gi[nt][hr * 2 + e]);
          }
      // H^H y: columns 0-1 (Y_hi) of lanes 4i plus columns 2-3 (Y_lo) of lanes 4i + 1
#pragma unroll
      for (int e = 0; e < 4; ++e) by[e] += __shfl_down_sync(0xffffffffu, by[e], 1);
      if ((lane & 3) == 0) {
        bv[gm] = make_float2(by[0], by[1]);
        bv[gm + 8] = make_float2(by[2], by[3]);
      }
      __syncwarp();
    }

    // ---------------- FP32 Cholesky solve, one element per half-warp (lane i: row i)
    const int jme = j0 + half;
    const bool valid = jme < nd;
    float2* G = Gs + half * MT * GS;
    float4* col = colb + half * MT;
    float2 a[MT];
#pragma unroll
    for (int jj = 0; jj < MT; ++jj) {
      a[jj] = G[row * GS + jj];
      if (jj == row) a[jj] = make_float2(a[jj].x + reg, 0.f);  // compile-time index: a[] stays in registers
    }
    float2 bi = bs[half * MT + row];
    float pmin = INFINITY, pmax = 0.f, inv_i = 0.f;
    bool ok = true;
    // right-looking Cholesky; column k of L goes through shared memory as (re, re, im, im)
    // so that each update a[jj] -= l_ik conj(l_jk) is two packed FMAs; every loop has a
    // fixed trip count so that a[] stays in registers
#pragma unroll
    for (int k = 0; k < MT; ++k) {
      const float dkk = __shfl_sync(0xffffffffu, a[k].x, k, 16);
      ok = ok && (dkk > 0.f);
      const float ik = rsqrtf(fmaxf(dkk, 1e-30f));
      const float pk = dkk * ik;
      pmin = fminf(pmin, pk);
      pmax = fmaxf(pmax, pk);
      if (row == k) inv_i = ik;
      const float2 lik = row > k ? cscale(a[k], ik) : (row == k ? make_float2(pk, 0.f) : make_float2(0.f, 0.f));
      a[k] = lik;
      col[row] = make_float4(lik.x, lik.x, lik.y, lik.y);
      __syncwarp();
      // (the predicate keeps the scheduler from hoisting every column load of the step:
      // without it the factorization spills)
      const float2 n0 = make_float2(-lik.x, -lik.y), n1 = make_float2(-lik.y, lik.x);
#pragma unroll
      for (int jj = 0; jj < MT; ++jj) {
        if (jj <= k) continue;
        const float4 c = col[jj];
        if (row >= jj) {
          a[jj] = __ffma2_rn(n0, make_float2(c.x, c.y), a[jj]);
          a[jj] = __ffma2_rn(n1, make_float2(c.z, c.w), a[jj]);
        }
      }
      __syncwarp();
    }
    // forward: L z = b (lane i holds row i of L). Every lane updates: L[i][k] = 0 for
    // i < k, and lane k's own value is not read after step k.
    float2 zi = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < MT; ++k) {
      const float2 zl = cscale(bi, inv_i);
      const float2 zk = make_float2(__shfl_sync(0xffffffffu, zl.x, k, 16), __shfl_sync(0xffffffffu, zl.y, k, 16));
      if (row == k) zi = zk;
      bi = csub(bi, cmul(a[k], zk));
    }
    // backward: L^H x = z with lane i holding column i of L (transposed through G):
    // once x_p is known every lane i < p subtracts conj(L[p][i]) x_p from its sum
#pragma unroll
    for (int p = 0; p < MT; ++p) G[row * GS + p] = a[p];
    __syncwarp();
#pragma unroll
    for (int p = 0; p < MT; ++p) a[p] = G[p * GS + row];
    float2 acc = make_float2(0.f, 0.f), xi = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = MT - 1; p >= 0; --p) {
      const float2 xl = cscale(csub(zi, acc), inv_i);
      const float2 xp = make_float2(__shfl_sync(0xffffffffu, xl.x, p, 16), __shfl_sync(0xffffffffu, xl.y, p, 16));
      if (row == p) xi = xp;
      acc = cadd(acc, cmulc(a[p], xp));  // L[p][i] = 0 for i > p; lane p's sum is not read after step p
    }
    __syncwarp();  // G reads done before the next element pair's Gram
    const bool cond_bad = !ok || pmax * pmax > kCondLimit * pmin * pmin;  // (pmax / pmin)^2 > 1e6
    const unsigned need = __ballot_sync(0xffffffffu, valid && cond_bad && row == 0);
    if (need) {
      // FP64 Gram and matched filter of the flagged elements from their channel
      // (lane i: row i), then a serial FP64 Cholesky solve on the half's first lane
      const bool mine = (need >> (16 * half)) & 1u;
      double2* G64 = reinterpret_cast<double2*>(Phi) + half * MT * MT;  // P tiles are free now
      double2* b64 = reinterpret_cast<double2*>(colb) + half * MT;      // so is the column broadcast
      if (mine) {
        const float2 gg = gsave[half];
        const int cc = csave[half];
        double2 bacc = make_double2(0.0, 0.0);
        for (int r = 0; r < NRX; ++r) {
          const float2 hi = cmul(make_float2(Sm[r * SMF + row], Sm[r * SMF + MT + row]), gg);
          const float2 yv = grid[(((int64_t)b * NRX + r) * W + w) * gcols + cc];
          bacc.x += (double)hi.x * yv.x + (double)hi.y * yv.y;  // conj(h) y
          bacc.y += (double)hi.x * yv.y - (double)hi.y * yv.x;
        }
        b64[row] = bacc;
        for (int jj = 0; jj <= row; ++jj) {
          double2 acc64 = make_double2(0.0, 0.0);
          for (int r = 0; r < NRX; ++r) {
            const float2 hi = cmul(make_float2(Sm[r * SMF + row], Sm[r * SMF + MT + row]), gg);
            const float2 hj = cmul(make_float2(Sm[r * SMF + jj], Sm[r * SMF + MT + jj]), gg);
            acc64.x += (double)hi.x * hj.x + (double)hi.y * hj.y;  // conj(h_i) h_j
            acc64.y += (double)hi.x * hj.y - (double)hi.y * hj.x;
          }
          G64[row * MT + jj] = acc64;
        }
      }
      __syncwarp();
      if (mine && row == 0) {
        float2 xo[MT];
        if (!solve_fp64(G64, b64, (double)reg, xo))
          for (int i = 0; i < MT; ++i) xo[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        for (int i = 0; i < MT; ++i) xs[half * MT + i] = xo[i];
      }
      __syncwarp();
      if (mine) xi = xs[half * MT + row];
      n64 += (row == 0 && mine) ? 1u : 0u;
    }
    if (valid) {
      bad = bad || !(fabsf(xi.x) < INFINITY && fabsf(xi.y) < INFINITY);
      const int64_t k = k0 + jme;
      const uint32_t rx_v = qam_decide(qt, xi);
      const uint32_t tx_v = element_bits(bc, seed, drop0 + b, (uint32_t)row, k * m, m);
      local += __popc(rx_v ^ tx_v);
      if (equalized) equalized[((int64_t)b * MT + row) * num_data + k] = xi;
    }
    __syncwarp();
  }
  // block totals
  for (int o = 16; o > 0; o >>= 1) {
    local += __shfl_down_sync(0xffffffffu, local, o);
    n64 += __shfl_down_sync(0xffffffffu, n64, o);
  }
  const bool any_bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    if (local) atomicAdd(errors + b, local);
    if (any_bad) atomicOr(errors + b, HPX_DROP_NUMERIC);
    if (n64 && fp64_count) atomicAdd(fp64_count + b, n64);
  }
}

template <int NRX>
hpx_status launch_massive(const hpx_fading* f, const void* state, const hpx_frame* fr, int mode, const hpx_cf32* grid,
                          int gcols, const float* nv, uint64_t seed, int64_t drop0, int B, uint32_t* errors,
                          uint32_t* fp64_count, hpx_cf32* equalized, cudaStream_t s) {
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const FadingConst fc = fading_const(f);
  const int C = fr->info.num_columns, m = fr->info.bits_per_symbol;
  const size_t smem = (size_t)MWARPS * MassiveSmem<NRX>::WARP_BYTES + (size_t)NRX * SMF * sizeof(float) +
                      (size_t)fc.L * sizeof(float2) * (1 + fc.S1) + (size_t)fc.L * sizeof(int);
  if (smem > 220 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: frame needs %zu bytes of shared memory", smem);
  auto kern = k_detect_massive<NRX>;
  HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 g(fr->info.num_words, B);
  kern<<<g, MWARPS * 32, smem, s>>>(fc, fading_view(f, state), fr->info.num_subcarriers, fr->info.num_words, C, m,
                                     fr->d_window_start, fr->d_data_offset, fr->d_num_data_word, fr->d_data_column,
                                     fr->d_bins, fr->d_twiddle, qt, mode, reinterpret_cast<const float2*>(grid), gcols,
                                     nv, seed, drop0, errors, fp64_count, reinterpret_cast<float2*>(equalized),
                                     fr->info.num_data);
  HPX_LAUNCHED("detect_massive");
  return HPX_OK;
}

}  // namespace

extern "C" hpx_status hpx_detect_massive(const hpx_fading* f, const void* state, const hpx_frame* fr, int32_t mode,
                                         const hpx_cf32* grid, int32_t gcols, const float* nv, uint64_t seed,
                                         int64_t drop0, int32_t B, uint32_t* errors, uint32_t* fp64_count,
                                         hpx_cf32* equalized, void* stream) {
  if (!f || !state || !fr || !grid || !errors) return hpx_fail(HPX_ERR_ARG, "detect_massive: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_massive: unknown mode");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "detect_massive: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_massive: bad drop range");
  if (gcols < fr->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "detect_massive: grid too narrow");
  if (f->ntx != MT) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: 16 transmit streams required (got %d)", f->ntx);
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_massive: batch above 65535 drops per call");
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  if (fp64_count) HPX_CUDA(cudaMemsetAsync(fp64_count, 0, sizeof(uint32_t) * B, s));
  switch (f->nrx) {
    case 16: return launch_massive<16>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    case 32: return launch_massive<32>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    case 64: return launch_massive<64>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: %d receive antennas not supported (16, 32, 64)", f->nrx);
  }
}
