// LDPC block codes: systematic encoder from the parity-check matrix and a batched
// belief-propagation decoder (flooding schedule, sum-product check update).
//
// Follows the interface of the reference's aff3ct wrapper (fec/aff3ct/ldpc.cpp:
// LDPCCoding(num_iterations, H, syndrome checking, min iterations), encode /
// decode of one block, hard input and hard output) with the published algorithms:
//   encoder  Gaussian elimination of H over GF(2) to reduced row-echelon form; the
//            non-pivot columns carry the K = N - rank data bits, each pivot
//            column the parity sum of its row over the data bits;
//   decoder  channel LLRs L_v (hard input: bit 0 -> +4, bit 1 -> -4, see kHardLlr), messages on
//            the edges of H; per iteration every check sends
//            m_cv = prod sign(m_v'c) * phi(sum phi(|m_v'c|)) over its other
//            variables (phi(x) = -log tanh(x / 2), phi = phi^-1), every variable
//            sends m_vc = L_v + sum of its other checks' messages and decides
//            on the total; with syndrome checking the decoder stops once H x = 0
//            and at least min_iterations have run.
// One group of threads (a warp for small codes, a CTA otherwise) decodes one
// code block with its messages in shared memory.
#include <algorithm>
#include <cstring>

#include "hpx_internal.cuh"

struct hpx_ldpc {
  int N = 0, M = 0, K = 0, E = 0, R = 0;  // R: rank of H (parity bits)
  int KW = 0;                             // 32-bit words of a packed data block
  int32_t* d_chk_ptr = nullptr;           // [M + 1] edges of check c (check order)
  int32_t* d_chk_var = nullptr;           // [E] variable of edge e
  int32_t* d_var_ptr = nullptr;           // [N + 1]
  int32_t* d_var_edge = nullptr;          // [E] edges of variable v
  int32_t* d_info = nullptr;              // [K] codeword position of data bit k
  int32_t* d_parity = nullptr;            // [R] codeword position of parity bit i
  uint32_t* d_rows = nullptr;             // [R][KW] parity bit i = parity(rows[i] & data)
  std::vector<int32_t> h_info;
};

namespace {

// Channel LLR magnitude of a hard input bit. The wrapper's hard-in decode converts bits
// to LLRs inside aff3ct (not part of the checkout); with magnitude 1 the sum-product
// decoder leaves single bit errors of the shipped (128, 64) code uncorrected, which
// the reference's LDPC test requires corrected; 4 (a binary symmetric channel with
// crossover ~1.8 %) corrects them.
constexpr float kHardLlr = 4.0f;

// phi(x) = -log(tanh(x / 2)) = log((e^x + 1) / (e^x - 1)), its own inverse; the
// argument is clamped to [1e-6, 30] (phi(1e-6) = 14.5, phi(30) ~ 1.9e-13).
__device__ __forceinline__ float bp_phi(float x) {
  x = fminf(fmaxf(x, 1e-6f), 30.0f);
  const float e = expf(x);
  return logf((e + 1.0f) / (e - 1.0f));
}

template <int G>
__device__ __forceinline__ void group_sync() {
  if (G <= 32) __syncwarp();
  else __syncthreads();
}

// One group of G threads per code block; `msg` holds 2 E floats (check->variable,
// variable->check), `llr` N floats, `hard` N bytes, per group.
template <int G>
__global__ void k_ldpc_decode(int N, int M, int K, int E, const int32_t* __restrict__ chk_ptr,
                              const int32_t* __restrict__ chk_var, const int32_t* __restrict__ var_ptr,
                              const int32_t* __restrict__ var_edge, const int32_t* __restrict__ info,
                              const uint8_t* __restrict__ code, const float* __restrict__ llr_in, int B,
                              int iterations, int syndrome, int min_iterations, uint8_t* __restrict__ data,
                              int32_t* __restrict__ used) {
  extern __shared__ float4 smem4[];
  constexpr int GPB = G >= 256 ? 1 : 256 / G;  // groups per block
  const int g = threadIdx.x / G, t = threadIdx.x - g * G;
  const int blk = blockIdx.x * GPB + g;
  const size_t per = (size_t)2 * E + N;  // floats per group
  float* c2v = reinterpret_cast<float*>(smem4) + g * per;
  float* v2c = c2v + E;
  float* L = v2c + E;
  uint8_t* hard = reinterpret_cast<uint8_t*>(reinterpret_cast<float*>(smem4) + GPB * per) + g * ((N + 15) & ~15);
  __shared__ int flag[GPB];
  const bool valid = blk < B;
  for (int v = t; v < N; v += G) {
    float l = 0.0f;
    if (valid) l = llr_in ? llr_in[(int64_t)blk * N + v] : (code[(int64_t)blk * N + v] ? -kHardLlr : kHardLlr);
    L[v] = l;
    hard[v] = l < 0.0f;
    for (int j = var_ptr[v]; j < var_ptr[v + 1]; ++j) v2c[var_edge[j]] = l;
  }
  group_sync<G>();
  int it = 0;
  for (; it < iterations; ++it) {
    // check update
    for (int c = t; c < M; c += G) {
      const int e0 = chk_ptr[c], e1 = chk_ptr[c + 1];
      float sum = 0.0f;
      uint32_t neg = 0;
      for (int e = e0; e < e1; ++e) {  // phi(|m|) parked in c2v for the second pass
        const float m = v2c[e];
        const float p = bp_phi(fabsf(m));
        c2v[e] = p;
        sum += p;
        neg ^= m < 0.0f;
      }
      for (int e = e0; e < e1; ++e) {
        const float m = v2c[e];
        const float mag = bp_phi(fmaxf(sum - c2v[e], 0.0f));
        c2v[e] = ((neg ^ (m < 0.0f)) ? -mag : mag);
      }
    }
    group_sync<G>();
    // variable update and decision
    for (int v = t; v < N; v += G) {
      const int j0 = var_ptr[v], j1 = var_ptr[v + 1];
      float tot = L[v];
      for (int j = j0; j < j1; ++j) tot += c2v[var_edge[j]];
      for (int j = j0; j < j1; ++j) {
        const int e = var_edge[j];
        v2c[e] = tot - c2v[e];
      }
      hard[v] = tot < 0.0f;
    }
    if (t == 0) flag[g] = 0;
    group_sync<G>();
    if (syndrome && it + 1 >= min_iterations) {
      for (int c = t; c < M; c += G) {
        uint32_t p = 0;
        for (int e = chk_ptr[c]; e < chk_ptr[c + 1]; ++e) p ^= hard[chk_var[e]];
        if (p) flag[g] = 1;
      }
      group_sync<G>();
      const bool done = flag[g] == 0;
      group_sync<G>();
      if (done) {
        ++it;
        break;
      }
    }
  }
  if (!valid) return;
  for (int k = t; k < K; k += G) data[(int64_t)blk * K + k] = hard[info[k]];
  if (used && t == 0) used[blk] = it;
}

// One thread per (block, codeword bit): data bits are copied to their positions,
// parity bits are the parity of a packed row of the reduced parity-check matrix
// AND the packed data block.
__global__ void k_ldpc_encode(int N, int K, int R, int KW, const int32_t* __restrict__ info,
                              const int32_t* __restrict__ parity, const uint32_t* __restrict__ rows,
                              const uint8_t* __restrict__ data, int B, uint8_t* __restrict__ code) {
  extern __shared__ uint32_t packed[];  // [KW] of this block
  const int blk = blockIdx.y;
  const uint8_t* d = data + (int64_t)blk * K;
  for (int w = threadIdx.x; w < KW; w += blockDim.x) {
    uint32_t word = 0;
    for (int j = 0; j < 32 && w * 32 + j < K; ++j) word |= (uint32_t)(d[w * 32 + j] & 1u) << j;
    packed[w] = word;
  }
  __syncthreads();
  uint8_t* c = code + (int64_t)blk * N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K + R; i += gridDim.x * blockDim.x) {
    if (i < K) {
      c[info[i]] = d[i] & 1u;
    } else {
      const int r = i - K;
      uint32_t p = 0;
      for (int w = 0; w < KW; ++w) p ^= __popc(rows[(size_t)r * KW + w] & packed[w]) & 1u;
      c[parity[r]] = (uint8_t)p;
    }
  }
}

template <typename T>
cudaError_t put(T** dst, const std::vector<T>& src) {
  *dst = nullptr;
  if (src.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), src.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void release(hpx_ldpc* l) {
  if (!l) return;
  void* p[] = {l->d_chk_ptr, l->d_chk_var, l->d_var_ptr, l->d_var_edge, l->d_info, l->d_parity, l->d_rows};
  for (void* q : p)
    if (q) cudaFree(q);
  delete l;
}

}  // namespace

extern "C" {

hpx_status hpx_ldpc_create(int32_t N, int32_t M, int32_t E, const int32_t* edge_var, const int32_t* edge_chk,
                           hpx_ldpc** out) {
  if (!out || !edge_var || !edge_chk) return hpx_fail(HPX_ERR_ARG, "ldpc: null argument");
  *out = nullptr;
  if (N < 2 || M < 1 || M >= N || E < 1) return hpx_fail(HPX_ERR_ARG, "ldpc: bad matrix size");
  std::vector<std::pair<int, int>> edges;  // (check, variable)
  for (int e = 0; e < E; ++e) {
    if (edge_var[e] < 0 || edge_var[e] >= N || edge_chk[e] < 0 || edge_chk[e] >= M)
      return hpx_fail(HPX_ERR_ARG, "ldpc: edge %d out of range", e);
    edges.emplace_back(edge_chk[e], edge_var[e]);
  }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  E = (int)edges.size();
  std::vector<int32_t> chk_ptr(M + 1, 0), chk_var(E), var_ptr(N + 1, 0), var_edge(E);
  for (int e = 0; e < E; ++e) {
    chk_ptr[edges[e].first + 1]++;
    chk_var[e] = edges[e].second;
    var_ptr[edges[e].second + 1]++;
  }
  for (int c = 0; c < M; ++c) chk_ptr[c + 1] += chk_ptr[c];
  for (int v = 0; v < N; ++v) var_ptr[v + 1] += var_ptr[v];
  {
    std::vector<int32_t> fill(var_ptr.begin(), var_ptr.end() - 1);
    for (int e = 0; e < E; ++e) var_edge[fill[edges[e].second]++] = e;
  }
  // reduced row-echelon form of H over GF(2), rows as packed 64-bit words
  const int NW = (N + 63) / 64;
  std::vector<uint64_t> h((size_t)M * NW, 0);
  for (const auto& ed : edges) h[(size_t)ed.first * NW + ed.second / 64] |= 1ull << (ed.second % 64);
  std::vector<int> pivot_col;
  int row = 0;
  for (int col = 0; col < N && row < M; ++col) {
    int sel = -1;
    for (int r = row; r < M; ++r)
      if (h[(size_t)r * NW + col / 64] >> (col % 64) & 1ull) {
        sel = r;
        break;
      }
    if (sel < 0) continue;
    if (sel != row)
      for (int w = 0; w < NW; ++w) std::swap(h[(size_t)sel * NW + w], h[(size_t)row * NW + w]);
    for (int r = 0; r < M; ++r)
      if (r != row && (h[(size_t)r * NW + col / 64] >> (col % 64) & 1ull))
        for (int w = 0; w < NW; ++w) h[(size_t)r * NW + w] ^= h[(size_t)row * NW + w];
    pivot_col.push_back(col);
    ++row;
  }
  const int R = (int)pivot_col.size(), K = N - R;
  std::vector<char> is_pivot(N, 0);
  for (int c : pivot_col) is_pivot[c] = 1;
  std::vector<int32_t> info, parity(pivot_col.begin(), pivot_col.end());
  for (int c = 0; c < N; ++c)
    if (!is_pivot[c]) info.push_back(c);
  const int KW = (K + 31) / 32;
  std::vector<uint32_t> rows((size_t)R * KW, 0);  // pivot bit = sum over data bits k of H_rref[i][info[k]]
  for (int i = 0; i < R; ++i)
    for (int k = 0; k < K; ++k)
      if (h[(size_t)i * NW + info[k] / 64] >> (info[k] % 64) & 1ull) rows[(size_t)i * KW + k / 32] |= 1u << (k % 32);
  hpx_ldpc* l = new hpx_ldpc();
  l->N = N;
  l->M = M;
  l->K = K;
  l->E = E;
  l->R = R;
  l->KW = KW;
  l->h_info = info;
  cudaError_t err;
  if ((err = put(&l->d_chk_ptr, chk_ptr)) != cudaSuccess || (err = put(&l->d_chk_var, chk_var)) != cudaSuccess ||
      (err = put(&l->d_var_ptr, var_ptr)) != cudaSuccess || (err = put(&l->d_var_edge, var_edge)) != cudaSuccess ||
      (err = put(&l->d_info, info)) != cudaSuccess || (err = put(&l->d_parity, parity)) != cudaSuccess ||
      (err = put(&l->d_rows, rows)) != cudaSuccess) {
    release(l);
    return hpx_cuda_status(err, "ldpc tables");
  }
  *out = l;
  return HPX_OK;
}

hpx_status hpx_ldpc_destroy(hpx_ldpc* code) {
  release(code);
  return HPX_OK;
}

hpx_status hpx_ldpc_info(const hpx_ldpc* code, int32_t* data_bits, int32_t* code_bits, int32_t* info_positions) {
  if (!code) return hpx_fail(HPX_ERR_ARG, "ldpc_info: null code");
  if (data_bits) *data_bits = code->K;
  if (code_bits) *code_bits = code->N;
  if (info_positions) std::memcpy(info_positions, code->h_info.data(), code->h_info.size() * sizeof(int32_t));
  return HPX_OK;
}

hpx_status hpx_ldpc_encode(const hpx_ldpc* code, const uint8_t* data, int32_t B, uint8_t* out, void* stream) {
  if (!code || (B > 0 && (!data || !out))) return hpx_fail(HPX_ERR_ARG, "ldpc_encode: null argument");
  if (B < 0 || B > 65535) return hpx_fail(HPX_ERR_ARG, "ldpc_encode: batch out of range (0..65535)");
  if (B == 0) return HPX_OK;
  const int threads = 128;
  const int gx = std::max(1, std::min(64, (code->N + threads - 1) / threads));
  k_ldpc_encode<<<dim3(gx, B), threads, (size_t)code->KW * 4, as_stream(stream)>>>(
      code->N, code->K, code->R, code->KW, code->d_info, code->d_parity, code->d_rows, data, B, out);
  HPX_LAUNCHED("ldpc_encode");
  return HPX_OK;
}

hpx_status hpx_ldpc_decode(const hpx_ldpc* code, const uint8_t* hard, const float* llr, int32_t B, int32_t iterations,
                           int32_t syndrome_checking, int32_t min_iterations, uint8_t* data, int32_t* iterations_used,
                           void* stream) {
  if (!code || (B > 0 && ((!hard && !llr) || !data))) return hpx_fail(HPX_ERR_ARG, "ldpc_decode: null argument");
  if (iterations < 1) return hpx_fail(HPX_ERR_ARG, "Number of decoding iterations must be greater than zero");
  if (B < 0) return hpx_fail(HPX_ERR_ARG, "ldpc_decode: negative batch");
  if (B == 0) return HPX_OK;
  const size_t per = ((size_t)2 * code->E + code->N) * sizeof(float) + (size_t)((code->N + 15) & ~15);
  cudaStream_t s = as_stream(stream);
  if (per * 8 <= 48 * 1024) {  // warp per code block, 8 per CTA
    const int blocks = (B + 7) / 8;
    k_ldpc_decode<32><<<blocks, 256, per * 8, s>>>(code->N, code->M, code->K, code->E, code->d_chk_ptr,
                                                    code->d_chk_var, code->d_var_ptr, code->d_var_edge, code->d_info,
                                                    hard, llr, B, iterations, syndrome_checking, min_iterations, data,
                                                    iterations_used);
  } else {
    if (per > 200 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "ldpc_decode: code too large for one CTA");
    if (per > 48 * 1024)
      HPX_CUDA(cudaFuncSetAttribute(k_ldpc_decode<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)per));
    k_ldpc_decode<256><<<B, 256, per, s>>>(code->N, code->M, code->K, code->E, code->d_chk_ptr, code->d_chk_var,
                                           code->d_var_ptr, code->d_var_edge, code->d_info, hard, llr, B, iterations,
                                           syndrome_checking, min_iterations, data, iterations_used);
  }
  HPX_LAUNCHED("ldpc_decode");
  return HPX_OK;
}

}  // extern "C"
