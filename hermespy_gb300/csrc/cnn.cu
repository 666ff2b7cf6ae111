// Learned channel estimator: a residual CNN that refines per-stream LS estimates
// of a MIMO grid into the full channel (no counterpart in the reference).
//
//   s  = RMS of the drop's LS estimate (per drop, over pairs, words and columns)
//   x0 = LS / s as 32 channels (16 antenna pairs x re/im) over (word, column)
//   h_l = relu(conv3x3_l(h_{l-1}) + b_l), l = 1..5;  out = LS + s (conv3x3_6(h_5) + b_6)
// so the network works at unit scale whatever the channel energy and SNR.
//
// Activations are BF16 NHWC ([drop][word][column][32 channels], 64 bytes per grid
// element); every layer is an implicit GEMM (M = grid elements, N = 32 output
// channels, K = 9 taps x 32 input channels) on the BF16 tensor cores with FP32
// accumulation (mma.sync m16n8k16). Training runs the same forward kernel, its
// transpose for the input gradients (weights flipped and transposed), a
// weight-gradient kernel and Adam on FP32 master weights.
#include <cuda_bf16.h>

#include <cmath>
#include <random>
#include <vector>

#include "hpx_internal.cuh"

namespace {

constexpr int CH = 32;          // channels of every layer
constexpr int KK = 9 * CH;      // GEMM depth: 3x3 taps x input channels
constexpr int LAYERS = 6;
constexpr int TH = 2, TW = 64;  // output tile (rows = words, columns)
constexpr int IN_H = TH + 2, IN_W = TW + 2, IN_PX = IN_H * IN_W;
constexpr int WPITCH = KK + 8;  // shared-memory weight row (bf16): 592 bytes, conflict-free ldmatrix
constexpr int NPAIR = CH / 2;   // antenna pairs carried by the 32 channels

// Byte offset of 16-byte chunk q (channels 8q..8q+7) of tile pixel pi: the chunk
// index is XOR-ed with bits 1-2 of the pixel, so 8 consecutive pixels of one chunk
// fall on 8 distinct 16-byte bank groups (ldmatrix without conflicts).
__device__ __forceinline__ int swz(int pi, int q) { return pi * 64 + ((q ^ ((pi >> 1) & 3)) << 4); }

__device__ __forceinline__ uint32_t bf2_bits(float lo, float hi) {
  const __nv_bfloat162 t = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &t, sizeof(u));
  return u;
}

// Store 16 packed bf16 pairs (64 bytes, one grid element) as four 16-byte stores.
__device__ __forceinline__ void store_px(__nv_bfloat16* dst, const uint32_t (&u)[NPAIR]) {
  uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = make_uint4(u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Load the (TH+2) x (TW+2) input tile with halo around output tile (h0, w0) of
// drop b into swizzled shared memory; elements outside the grid read as zero.
__device__ __forceinline__ void load_tile(unsigned char* sm, const __nv_bfloat16* __restrict__ act, int b, int H, int W,
                                          int h0, int w0) {
  for (int q = threadIdx.x; q < IN_PX * 4; q += blockDim.x) {
    const int pi = q >> 2, ch = q & 3;
    const int ty = pi / IN_W, tx = pi - ty * IN_W;
    const int h = h0 - 1 + ty, w = w0 - 1 + tx;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (h >= 0 && h < H && w >= 0 && w < W)
      v = __ldg(reinterpret_cast<const uint4*>(act + (((int64_t)b * H + h) * W + w) * CH) + ch);
    *reinterpret_cast<uint4*>(sm + swz(pi, ch)) = v;
  }
}

// EPI 0: + bias, ReLU -> bf16 NHWC.  EPI 1: + bias + residual (complex planes)
// -> complex planes [drop][pair][word][ccols].  EPI 2: times (mask > 0) -> bf16
// NHWC (input gradient through the previous layer's ReLU).
template <int EPI>
__global__ void __launch_bounds__(128) k_conv3x3(int H, int W, const __nv_bfloat16* __restrict__ in,
                                                 const __nv_bfloat16* __restrict__ wt, const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ out, const __nv_bfloat16* __restrict__ mask,
                                                 const float2* __restrict__ resid, float2* __restrict__ out_c,
                                                 int ccols, const float* __restrict__ pw, float inv_count) {
  __shared__ __align__(128) unsigned char s_in[IN_PX * 64];
  __shared__ __align__(128) __nv_bfloat16 s_w[CH * WPITCH];
  const int tiles_w = (W + TW - 1) / TW;
  const int tile = blockIdx.x, b = blockIdx.y;
  const int h0 = (tile / tiles_w) * TH, w0 = (tile - (tile / tiles_w) * tiles_w) * TW;
  for (int q = threadIdx.x; q < CH * (KK / 8); q += blockDim.x) {
    const int n = q / (KK / 8), c16 = q - n * (KK / 8);
    *reinterpret_cast<uint4*>(s_w + n * WPITCH + c16 * 8) = __ldg(reinterpret_cast<const uint4*>(wt + n * KK) + c16);
  }
  load_tile(s_in, in, b, H, W, h0, w0);
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ty = warp >> 1, tx0 = (warp & 1) * 32;
  const int j = lane >> 3, r = lane & 7;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.f;
  const uint32_t in_base = smem_u32(s_in), w_base = smem_u32(s_w);
#pragma unroll 1
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3, dx = tap - dy * 3;
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
      uint32_t bf[4][2];
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int n = half * 16 + (j >> 1) * 8 + r;
        const int k = tap * CH + kc * 16 + (j & 1) * 8;
        uint32_t r0, r1, r2, r3;
        ldsm_x4(w_base + (n * WPITCH + k) * 2, r0, r1, r2, r3);
        bf[half * 2][0] = r0;
        bf[half * 2][1] = r1;
        bf[half * 2 + 1][0] = r2;
        bf[half * 2 + 1][1] = r3;
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int pi = (ty + dy) * IN_W + tx0 + mt * 16 + (j & 1) * 8 + r + dx;
        uint32_t a[4];
        ldsm_x4(in_base + swz(pi, kc * 2 + (j >> 1)), a[0], a[1], a[2], a[3]);
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], a, bf[nt][0], bf[nt][1]);
      }
    }
  }

  const int h = h0 + ty;
  if (h >= H) return;
  const int g = lane >> 2, cq = (lane & 3) * 2;
  const float scale = EPI == 1 ? sqrtf(pw[b] * inv_count) : 1.f;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hr = 0; hr < 2; ++hr) {
      const int w = w0 + tx0 + mt * 16 + g + hr * 8;
      if (w >= W) continue;
      const int64_t px = ((int64_t)b * H + h) * W + w;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + cq;
        float v0 = acc[mt][nt][hr * 2], v1 = acc[mt][nt][hr * 2 + 1];
        if (EPI == 0) {
          v0 = fmaxf(v0 + bias[n], 0.f);
          v1 = fmaxf(v1 + bias[n + 1], 0.f);
          *reinterpret_cast<__nv_bfloat162*>(out + px * CH + n) = __floats2bfloat162_rn(v0, v1);
        } else if (EPI == 1) {
          const int64_t e = (((int64_t)b * NPAIR + (n >> 1)) * H + h) * ccols + w;
          const float2 x = resid[e];
          out_c[e] = make_float2(fmaf(scale, v0 + bias[n], x.x), fmaf(scale, v1 + bias[n + 1], x.y));
        } else {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + px * CH + n);
          v0 = __low2float(mk) > 0.f ? v0 : 0.f;
          v1 = __high2float(mk) > 0.f ? v1 : 0.f;
          *reinterpret_cast<__nv_bfloat162*>(out + px * CH + n) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
}

// Weight and bias gradients of one layer: dW[n][tap*32 + c] += sum_p dY[p][n] X[p + tap][c],
// db[n] += sum_p dY[p][n] over all grid elements of the batch. Nine warps, warp = tap;
// each block walks a contiguous range of tiles and adds its partial sums once.
__global__ void __launch_bounds__(288) k_conv3x3_wgrad(int H, int W, int B, const __nv_bfloat16* __restrict__ x,
                                                       const __nv_bfloat16* __restrict__ dy, float* __restrict__ dw,
                                                       float* __restrict__ db) {
  __shared__ __align__(128) unsigned char s_x[IN_PX * 64];
  __shared__ __align__(128) unsigned char s_d[TH * TW * 64];
  const int tiles_w = (W + TW - 1) / TW, tiles_h = (H + TH - 1) / TH;
  const int64_t tiles = (int64_t)B * tiles_h * tiles_w;
  const int64_t per = (tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * per, t1 = min(tiles, t0 + per);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tap = warp, ddy = tap / 3, ddx = tap - ddy * 3;
  const int j = lane >> 3, r = lane & 7;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.f;
  float bsum = 0.f;
  const uint32_t xb = smem_u32(s_x), dbase = smem_u32(s_d);
  for (int64_t t = t0; t < t1; ++t) {
    const int b = (int)(t / (tiles_h * tiles_w));
    const int rem = (int)(t - (int64_t)b * tiles_h * tiles_w);
    const int h0 = (rem / tiles_w) * TH, w0 = (rem - (rem / tiles_w) * tiles_w) * TW;
    __syncthreads();  // previous tile consumed
    load_tile(s_x, x, b, H, W, h0, w0);
    for (int q = threadIdx.x; q < TH * TW * 4; q += blockDim.x) {
      const int pd = q >> 2, ch = q & 3;
      const int ty = pd / TW, tx = pd - ty * TW;
      const int h = h0 + ty, w = w0 + tx;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (h < H && w < W) v = __ldg(reinterpret_cast<const uint4*>(dy + (((int64_t)b * H + h) * W + w) * CH) + ch);
      *reinterpret_cast<uint4*>(s_d + swz(pd, ch)) = v;
    }
    __syncthreads();
    if (threadIdx.x < CH) {
      const __nv_bfloat16* sd = reinterpret_cast<const __nv_bfloat16*>(s_d);
      const int n = threadIdx.x, q = n >> 3, e = n & 7;
      for (int pd = 0; pd < TH * TW; ++pd) bsum += __bfloat162float(sd[swz(pd, q) / 2 + e]);
    }
#pragma unroll
    for (int ty = 0; ty < TH; ++ty)
#pragma unroll 1
      for (int ks = 0; ks < TW / 16; ++ks) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int pd = ty * TW + ks * 16 + (j >> 1) * 8 + r;
          ldsm_x4_t(dbase + swz(pd, mt * 2 + (j & 1)), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
        }
        uint32_t bf[4][2];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int pi = (ty + ddy) * IN_W + ks * 16 + (j & 1) * 8 + r + ddx;
          uint32_t r0, r1, r2, r3;
          ldsm_x4_t(xb + swz(pi, half * 2 + (j >> 1)), r0, r1, r2, r3);
          bf[half * 2][0] = r0;
          bf[half * 2][1] = r1;
          bf[half * 2 + 1][0] = r2;
          bf[half * 2 + 1][1] = r3;
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], a[mt], bf[nt][0], bf[nt][1]);
      }
  }
  const int g = lane >> 2, cq = (lane & 3) * 2;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int n = mt * 16 + g + (i >> 1) * 8;
        const int c = nt * 8 + cq + (i & 1);
        atomicAdd(dw + n * KK + tap * CH + c, acc[mt][nt][i]);
      }
  if (threadIdx.x < CH) atomicAdd(db + threadIdx.x, bsum);
}

// Per drop: pw[b] = sum of |LS|^2 over pairs, words and columns (blockIdx.y = drop).
__global__ void k_cnn_power(int H, int W, int ccols, const float2* __restrict__ csi, float* __restrict__ pw) {
  const int b = blockIdx.y;
  const int total = NPAIR * H * W;
  float e = 0.f;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int p = q / (H * W), rem = q - p * H * W, h = rem / W, w = rem - h * W;
    const float2 z = csi[(((int64_t)b * NPAIR + p) * H + h) * ccols + w];
    e = fmaf(z.x, z.x, fmaf(z.y, z.y, e));
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(pw + b, e);
}

// complex planes [drop][pair][word][ccols] / s -> bf16 NHWC [drop][word][column][32]
__global__ void k_cnn_pack(int H, int W, int ccols, int B, const float2* __restrict__ csi, const float* __restrict__ pw,
                           float inv_count, __nv_bfloat16* __restrict__ out) {
  const int64_t total = (int64_t)B * H * W;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / ((int64_t)H * W);
    const int rem = (int)(q - b * H * W);
    const int h = rem / W, w = rem - h * W;
    const float is = rsqrtf(fmaxf(pw[b] * inv_count, 1e-30f));
    uint32_t v[NPAIR];
#pragma unroll
    for (int p = 0; p < NPAIR; ++p) {
      const float2 z = csi[((b * NPAIR + p) * H + h) * ccols + w];
      v[p] = bf2_bits(z.x * is, z.y * is);
    }
    store_px(out + q * CH, v);
  }
}

// dY = (out - truth) / s as bf16 NHWC and the batch's sum of |out - truth|^2 / s^2
// (the loss at the network's unit scale).
__global__ void k_cnn_loss_grad(int H, int W, int ccols, int B, const float2* __restrict__ outc,
                                const float2* __restrict__ truth, const float* __restrict__ pw, float inv_count,
                                __nv_bfloat16* __restrict__ dy, double* __restrict__ loss) {
  const int64_t total = (int64_t)B * H * W;
  float e = 0.f;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / ((int64_t)H * W);
    const int rem = (int)(q - b * H * W);
    const int h = rem / W, w = rem - h * W;
    const float is = rsqrtf(fmaxf(pw[b] * inv_count, 1e-30f));
    uint32_t v[NPAIR];
#pragma unroll
    for (int p = 0; p < NPAIR; ++p) {
      const int64_t i = ((b * NPAIR + p) * H + h) * ccols + w;
      const float2 o = outc[i], t = truth[i];
      const float dx = (o.x - t.x) * is, dyv = (o.y - t.y) * is;
      e = fmaf(dx, dx, fmaf(dyv, dyv, e));
      v[p] = bf2_bits(dx, dyv);
    }
    store_px(dy + q * CH, v);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)e);
}

// Adam on the FP32 master parameters; refreshes the BF16 forward weights and the
// flipped, transposed copies used for input gradients:
//   wd[l][c][(8 - tap) * 32 + n] = w[l][n][tap * 32 + c].
__global__ void k_cnn_adam(int nparam, float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1, float c2,
                           float gscale, __nv_bfloat16* __restrict__ wbf, __nv_bfloat16* __restrict__ wdf) {
  const int nw = LAYERS * CH * KK;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nparam; i += gridDim.x * blockDim.x) {
    const float g = grad[i] * gscale;
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    if (i < nw) {
      const int l = i / (CH * KK), rem = i - l * CH * KK;
      const int n = rem / KK, k = rem - n * KK, tap = k / CH, c = k - tap * CH;
      wbf[i] = __float2bfloat16_rn(pi);
      wdf[(size_t)l * CH * KK + c * KK + (8 - tap) * CH + n] = __float2bfloat16_rn(pi);
    }
  }
}

}  // namespace

struct hpx_cnn {
  int H = 0, W = 0, max_batch = 0;
  int64_t step = 0;
  // parameters: weights [6][32][288] then biases [6][32] (FP32 master, Adam state, gradients)
  float* d_param = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  float* d_grad = nullptr;
  __nv_bfloat16* d_w = nullptr;   // [6][32][288]
  __nv_bfloat16* d_wd = nullptr;  // [6][32][288] flipped / transposed
  __nv_bfloat16* d_act = nullptr; // [6][max_batch][H][W][32]: x0, h1..h5
  __nv_bfloat16* d_g = nullptr;   // [2][max_batch][H][W][32] gradient ping-pong
  float2* d_out = nullptr;        // [max_batch][16][H][W] training output
  float* d_pw = nullptr;          // [max_batch] per-drop LS power sums
  double* d_loss = nullptr;
};

namespace {

constexpr int NW = LAYERS * CH * KK, NB = LAYERS * CH, NPARAM = NW + NB;

void cnn_release(hpx_cnn* c) {
  if (!c) return;
  void* p[] = {c->d_param, c->d_m, c->d_v, c->d_grad, c->d_w, c->d_wd, c->d_act, c->d_g, c->d_out, c->d_pw, c->d_loss};
  for (void* q : p)
    if (q) cudaFree(q);
  delete c;
}

hpx_status refresh_bf16(hpx_cnn* c) {
  // an Adam step with zero learning rate and zero gradient rewrites both bf16 copies
  HPX_CUDA(cudaMemset(c->d_grad, 0, sizeof(float) * NPARAM));
  std::vector<float> zero(NPARAM, 0.f);
  float* tmp_m = nullptr;
  float* tmp_v = nullptr;
  HPX_CUDA(cudaMalloc(&tmp_m, sizeof(float) * NPARAM));
  HPX_CUDA(cudaMalloc(&tmp_v, sizeof(float) * NPARAM));
  cudaMemset(tmp_m, 0, sizeof(float) * NPARAM);
  cudaMemset(tmp_v, 0, sizeof(float) * NPARAM);
  k_cnn_adam<<<(NPARAM + 255) / 256, 256>>>(NPARAM, c->d_param, tmp_m, tmp_v, c->d_grad, 0.f, 0.9f, 0.999f, 1e-8f,
                                             1.f, 1.f, 1.f, c->d_w, c->d_wd);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(tmp_m);
  cudaFree(tmp_v);
  if (e != cudaSuccess) return hpx_cuda_status(e, "cnn weights");
  return HPX_OK;
}

int conv_tiles(int H, int W) { return ((H + TH - 1) / TH) * ((W + TW - 1) / TW); }

// Power sums and the packed, scaled input of B drops of complex planes.
hpx_status prepare(const hpx_cnn* c, int B, const float2* csi, int ccols, __nv_bfloat16* x0, cudaStream_t s) {
  HPX_CUDA(cudaMemsetAsync(c->d_pw, 0, sizeof(float) * B, s));
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  k_cnn_power<<<dim3(16, B), 256, 0, s>>>(c->H, c->W, ccols, csi, c->d_pw);
  HPX_LAUNCHED("cnn power");
  const int64_t px = (int64_t)B * c->H * c->W;
  k_cnn_pack<<<(int)((px + 255) / 256), 256, 0, s>>>(c->H, c->W, ccols, B, csi, c->d_pw, inv, x0);
  HPX_LAUNCHED("cnn pack");
  return HPX_OK;
}

hpx_status forward(const hpx_cnn* c, int B, const __nv_bfloat16* x0, __nv_bfloat16* const* act_out,
                   const float2* resid, float2* out_c, int ccols, cudaStream_t s) {
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  dim3 g(conv_tiles(c->H, c->W), B);
  const __nv_bfloat16* in = x0;
  for (int l = 0; l < LAYERS - 1; ++l) {
    k_conv3x3<0><<<g, 128, 0, s>>>(c->H, c->W, in, c->d_w + (size_t)l * CH * KK, c->d_param + NW + l * CH,
                                   act_out[l], nullptr, nullptr, nullptr, 0, nullptr, 0.f);
    in = act_out[l];
  }
  k_conv3x3<1><<<g, 128, 0, s>>>(c->H, c->W, in, c->d_w + (size_t)(LAYERS - 1) * CH * KK,
                                 c->d_param + NW + (LAYERS - 1) * CH, nullptr, nullptr, resid, out_c, ccols, c->d_pw,
                                 inv);
  HPX_LAUNCHED("cnn forward");
  return HPX_OK;
}

}  // namespace

extern "C" {

hpx_status hpx_cnn_create(int32_t num_words, int32_t num_columns, int32_t max_batch, const float* params,
                          uint64_t seed, hpx_cnn** out) {
  if (!out) return hpx_fail(HPX_ERR_ARG, "cnn: null argument");
  *out = nullptr;
  if (num_words < 1 || num_columns < 1 || max_batch < 1 || max_batch > 65535)
    return hpx_fail(HPX_ERR_ARG, "cnn: bad grid or batch size");
  hpx_cnn* c = new hpx_cnn();
  c->H = num_words;
  c->W = num_columns;
  c->max_batch = max_batch;
  std::vector<float> host(NPARAM, 0.f);
  if (params) {
    host.assign(params, params + NPARAM);
  } else {
    // He-normal convolutions; the last layer starts near zero so the network
    // starts as the identity on its LS input.
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / KK));
    for (int l = 0; l < LAYERS; ++l)
      for (int i = 0; i < CH * KK; ++i) host[(size_t)l * CH * KK + i] = nd(rng) * (l == LAYERS - 1 ? 0.01f : 1.f);
  }
  const size_t act = (size_t)max_batch * num_words * num_columns * CH;
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_param, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_m, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_v, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_grad, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_w, sizeof(__nv_bfloat16) * NW)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_wd, sizeof(__nv_bfloat16) * NW)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_act, sizeof(__nv_bfloat16) * act * LAYERS)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_g, sizeof(__nv_bfloat16) * act * 2)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_out, sizeof(float2) * (size_t)max_batch * NPAIR * num_words * num_columns)) !=
          cudaSuccess ||
      (e = cudaMalloc(&c->d_loss, sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_pw, sizeof(float) * max_batch)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_param, host.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(c->d_m, 0, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMemset(c->d_v, 0, sizeof(float) * NPARAM)) != cudaSuccess) {
    cnn_release(c);
    return hpx_cuda_status(e, "cnn buffers");
  }
  const hpx_status st = refresh_bf16(c);
  if (st != HPX_OK) {
    cnn_release(c);
    return st;
  }
  *out = c;
  return HPX_OK;
}

hpx_status hpx_cnn_destroy(hpx_cnn* c) {
  cnn_release(c);
  return HPX_OK;
}

int32_t hpx_cnn_num_params(void) { return NPARAM; }

hpx_status hpx_cnn_get_params(const hpx_cnn* c, float* params) {
  if (!c || !params) return hpx_fail(HPX_ERR_ARG, "cnn_get_params: null argument");
  HPX_CUDA(cudaMemcpy(params, c->d_param, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return HPX_OK;
}

hpx_status hpx_cnn_get_grads(const hpx_cnn* c, float* grads) {
  if (!c || !grads) return hpx_fail(HPX_ERR_ARG, "cnn_get_grads: null argument");
  HPX_CUDA(cudaMemcpy(grads, c->d_grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return HPX_OK;
}

hpx_status hpx_cnn_refine(const hpx_cnn* c, hpx_cf32* csi, int32_t ccols, int32_t B, void* stream) {
  if (!c || !csi) return hpx_fail(HPX_ERR_ARG, "cnn_refine: null argument");
  if (B < 0) return hpx_fail(HPX_ERR_ARG, "cnn_refine: negative batch");
  if (ccols < c->W) return hpx_fail(HPX_ERR_SHAPE, "cnn_refine: CSI narrower than the network's grid");
  cudaStream_t s = as_stream(stream);
  const size_t act = (size_t)c->max_batch * c->H * c->W * CH;
  for (int b0 = 0; b0 < B; b0 += c->max_batch) {
    const int n = B - b0 < c->max_batch ? B - b0 : c->max_batch;
    float2* cs = reinterpret_cast<float2*>(csi) + (size_t)b0 * NPAIR * c->H * ccols;
    __nv_bfloat16* x0 = c->d_act;
    __nv_bfloat16* pp[2] = {c->d_g, c->d_g + act};
    __nv_bfloat16* outs[LAYERS - 1] = {pp[0], pp[1], pp[0], pp[1], pp[0]};
    HPX_TRY(prepare(c, n, cs, ccols, x0, s));
    HPX_TRY(forward(c, n, x0, outs, cs, cs, ccols, s));
  }
  return HPX_OK;
}

hpx_status hpx_cnn_train_step(hpx_cnn* c, const hpx_cf32* ls, const hpx_cf32* truth, int32_t ccols, int32_t B,
                              float lr, double* loss, void* stream) {
  if (!c || !ls || !truth) return hpx_fail(HPX_ERR_ARG, "cnn_train_step: null argument");
  if (B < 1 || B > c->max_batch) return hpx_fail(HPX_ERR_ARG, "cnn_train_step: batch must be in [1, %d]", c->max_batch);
  if (ccols != c->W) return hpx_fail(HPX_ERR_SHAPE, "cnn_train_step: CSI columns must equal the network's grid width");
  cudaStream_t s = as_stream(stream);
  const size_t act = (size_t)c->max_batch * c->H * c->W * CH;
  __nv_bfloat16* a[LAYERS];
  for (int l = 0; l < LAYERS; ++l) a[l] = c->d_act + act * l;
  const int64_t px = (int64_t)B * c->H * c->W;
  const int blocks = (int)((px + 255) / 256);
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  HPX_TRY(prepare(c, B, reinterpret_cast<const float2*>(ls), ccols, a[0], s));
  HPX_TRY(forward(c, B, a[0], a + 1, reinterpret_cast<const float2*>(ls), c->d_out, ccols, s));
  HPX_CUDA(cudaMemsetAsync(c->d_loss, 0, sizeof(double), s));
  __nv_bfloat16* g[2] = {c->d_g, c->d_g + act};
  k_cnn_loss_grad<<<blocks, 256, 0, s>>>(c->H, c->W, ccols, B, c->d_out, reinterpret_cast<const float2*>(truth),
                                         c->d_pw, inv, g[0], c->d_loss);
  HPX_LAUNCHED("cnn loss");
  HPX_CUDA(cudaMemsetAsync(c->d_grad, 0, sizeof(float) * NPARAM, s));
  const int tiles = B * conv_tiles(c->H, c->W);
  const int wblocks = tiles < 4 * 152 ? tiles : 4 * 152;
  dim3 gd(conv_tiles(c->H, c->W), B);
  int cur = 0;
  for (int l = LAYERS - 1; l >= 0; --l) {
    k_conv3x3_wgrad<<<wblocks, 288, 0, s>>>(c->H, c->W, B, a[l], g[cur], c->d_grad + (size_t)l * CH * KK,
                                            c->d_grad + NW + l * CH);
    HPX_LAUNCHED("cnn wgrad");
    if (l > 0) {
      k_conv3x3<2><<<gd, 128, 0, s>>>(c->H, c->W, g[cur], c->d_wd + (size_t)l * CH * KK, nullptr, g[cur ^ 1], a[l],
                                      nullptr, nullptr, 0, nullptr, 0.f);
      HPX_LAUNCHED("cnn dgrad");
      cur ^= 1;
    }
  }
  c->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)c->step)), c2 = 1.f / (1.f - std::pow(b2, (float)c->step));
  // gradients are sums over the batch's grid elements and channels: average them
  const float gscale = 1.f / (float)(px * CH);
  k_cnn_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(NPARAM, c->d_param, c->d_m, c->d_v, c->d_grad, lr, b1, b2, 1e-8f, c1,
                                                   c2, gscale, c->d_w, c->d_wd);
  HPX_LAUNCHED("cnn adam");
  if (loss) HPX_CUDA(cudaMemcpyAsync(loss, c->d_loss, sizeof(double), cudaMemcpyDeviceToDevice, s));
  return HPX_OK;
}

}  // extern "C"
