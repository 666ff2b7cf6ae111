// Frame layout tables and the library's error state.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>

#include "hpx_internal.cuh"

// ------------------------------------------------------------------ errors

static thread_local std::string g_last_error;

hpx_status hpx_fail(hpx_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

hpx_status hpx_cuda_status(cudaError_t err, const char* what) {
  return hpx_fail(HPX_ERR_CUDA, "CUDA error %d (%s) in %s", (int)err, cudaGetErrorString(err), what);
}

template <typename T>
static hpx_status upload(T** dst, const std::vector<T>& src) {
  if (src.empty()) {
    *dst = nullptr;
    return HPX_OK;
  }
  HPX_CUDA(cudaMalloc(reinterpret_cast<void**>(dst), src.size() * sizeof(T)));
  HPX_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return HPX_OK;
}

static void release(hpx_frame* f) {
  if (!f) return;
  void* ptrs[] = {f->d_prefix, f->d_zero_prefix, f->d_word_start, f->d_window_start, f->d_data_offset,
                  f->d_num_data_word, f->d_kind, f->d_index, f->d_bins, f->d_data_column, f->d_data_word,
                  f->d_twiddle, f->d_stage_twiddle, f->d_pilots, f->d_bin_code, f->d_constellation,
                  f->d_tx_src, f->d_tx_regular, f->d_tx_bitoff, f->d_constellation_lsb};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete f;
}

extern "C" {

int hpx_version(void) { return 10000; }

const char* hpx_last_error(void) { return g_last_error.c_str(); }

hpx_status hpx_drop_status(const uint32_t* errors, int64_t num_drops) {
  if (num_drops < 0 || (num_drops > 0 && !errors)) return hpx_fail(HPX_ERR_ARG, "drop_status: bad arguments");
  int64_t first_numeric = -1;
  for (int64_t i = 0; i < num_drops; ++i) {
    if (errors[i] & HPX_DROP_TIMEOUT)
      return hpx_fail(HPX_ERR_TIMEOUT, "drop %lld: a bounded tensor-core wait ran out (result invalid)", (long long)i);
    if ((errors[i] & HPX_DROP_NUMERIC) && first_numeric < 0) first_numeric = i;
  }
  if (first_numeric >= 0)
    return hpx_fail(HPX_ERR_NUMERIC, "drop %lld: non-finite pivot in the equalizer (NaN or inf channel, samples or "
                    "noise power)", (long long)first_numeric);
  return HPX_OK;
}

hpx_status hpx_frame_create(const hpx_frame_desc* desc, hpx_frame** out) {
  if (!desc || !out) return hpx_fail(HPX_ERR_ARG, "frame: null argument");
  *out = nullptr;
  const int N = desc->num_subcarriers;
  if (N < 64 || N > 4096 || (N & (N - 1)))
    return hpx_fail(HPX_ERR_UNSUPPORTED, "frame: number of subcarriers must be a power of two in [64, 4096] (got %d)", N);
  const int W = desc->num_words, C = desc->num_columns;
  if (W < 1) return hpx_fail(HPX_ERR_ARG, "frame: at least one word required");
  if (C < 1 || C > N) return hpx_fail(HPX_ERR_ARG, "frame: num_columns must be in [1, N]");
  int m;
  HPX_TRY(qam_bits_per_symbol(desc->modulation_order, &m));
  if (!desc->prefix || !desc->kind) return hpx_fail(HPX_ERR_ARG, "frame: null table");

  hpx_frame* f = new hpx_frame();
  f->dc_suppression = desc->dc_suppression ? 1 : 0;
  if (desc->pilot_comb < 0 || desc->pilot_comb > 64) {
    delete f;
    return hpx_fail(HPX_ERR_ARG, "frame: pilot_comb must be in [0, 64] (got %d)", desc->pilot_comb);
  }
  f->pilot_comb = desc->pilot_comb;
  f->h_prefix.assign(desc->prefix, desc->prefix + W);
  f->h_zero_prefix.assign(W, 0);
  if (desc->zero_prefix) f->h_zero_prefix.assign(desc->zero_prefix, desc->zero_prefix + W);
  f->h_kind.assign(desc->kind, desc->kind + (size_t)W * C);
  f->h_index.assign((size_t)W * C, -1);
  f->h_word_start.resize(W);
  f->h_window_start.resize(W);
  f->h_data_offset.resize(W);
  f->h_ref_offset.resize(W);
  std::vector<int32_t> num_data_word(W, 0), data_column, data_word;
  int64_t start = 0;
  int nd = 0, nr = 0;
  for (int w = 0; w < W; ++w) {
    const int p = f->h_prefix[w];
    if (p < 0 || p > N) {
      release(f);
      return hpx_fail(HPX_ERR_ARG, "frame: prefix length of word %d out of range", w);
    }
    f->h_word_start[w] = (int32_t)start;
    f->h_window_start[w] = (int32_t)(start + p);
    f->h_data_offset[w] = nd;
    f->h_ref_offset[w] = nr;
    for (int c = 0; c < C; ++c) {
      const int8_t k = f->h_kind[(size_t)w * C + c];
      if (k == HPX_RE_DATA) {
        f->h_index[(size_t)w * C + c] = nd++;
        data_column.push_back(c);
        data_word.push_back(w);
        num_data_word[w]++;
      } else if (k == HPX_RE_REFERENCE) {
        f->h_index[(size_t)w * C + c] = nr++;
      } else if (k != HPX_RE_NULL) {
        release(f);
        return hpx_fail(HPX_ERR_ARG, "frame: unknown element type %d", (int)k);
      }
    }
    start += p + N;
  }
  if (start > (1ll << 30)) {
    release(f);
    return hpx_fail(HPX_ERR_ARG, "frame: too many samples");
  }
  f->info.num_subcarriers = N;
  f->info.num_words = W;
  f->info.num_columns = C;
  f->info.modulation_order = desc->modulation_order;
  f->info.bits_per_symbol = m;
  f->info.num_data = nd;
  f->info.num_refs = nr;
  f->info.samples_per_frame = (int32_t)start;
  for (int w = 0; w < W; ++w) f->max_data_word = std::max(f->max_data_word, num_data_word[w]);

  // grid column -> FFT bin (ofdm.py:116-128 and 146-151)
  f->h_bins.resize(N);
  for (int c = 0; c < N; ++c) {
    int b;
    if (f->dc_suppression) b = c < N / 2 ? c + N / 2 : (c < N - 1 ? c + 1 - N / 2 : 0);
    else b = (c + N / 2) % N;
    f->h_bins[c] = b;
  }
  std::vector<float2> tw(N);
  for (int t = 0; t < N; ++t) {
    const double a = -2.0 * M_PI * (double)t / (double)N;
    tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  // Stockham stage twiddles of the OFDM FFT plans (radices per N as in fft.cuh):
  // stage with span Ns and radix R stores exp(-2 pi i r k / (Ns R)) at r Ns + k.
  std::vector<float2> stw(2 * (size_t)N, make_float2(1.f, 0.f));
  {
    int radix[3] = {0, 0, 0}, stages = 2;
    switch (N) {
      case 64: radix[0] = 8; radix[1] = 8; break;
      case 128: radix[0] = 16; radix[1] = 8; break;
      case 256: radix[0] = 16; radix[1] = 16; break;
      case 512: radix[0] = 16; radix[1] = 16; radix[2] = 2; stages = 3; break;
      case 1024: radix[0] = 16; radix[1] = 16; radix[2] = 4; stages = 3; break;
      case 2048: radix[0] = 16; radix[1] = 16; radix[2] = 8; stages = 3; break;
      default: radix[0] = 16; radix[1] = 16; radix[2] = 16; stages = 3; break;  // 4096
    }
    size_t off = 0;
    int Ns = radix[0];
    for (int st = 1; st < stages; ++st) {
      const int R = radix[st];
      for (int r = 0; r < R; ++r)
        for (int k = 0; k < Ns; ++k) {
          const double a = -2.0 * M_PI * (double)r * (double)k / ((double)Ns * R);
          stw[off + (size_t)r * Ns + k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
      off += (size_t)R * Ns;
      Ns *= R;
    }
  }
  std::vector<float2> pilots(nr);
  for (int k = 0; k < nr; ++k) pilots[k] = qam_symbol(desc->modulation_order, (uint32_t)(k % desc->modulation_order));
  std::vector<float2> constellation(desc->modulation_order);
  for (int v = 0; v < desc->modulation_order; ++v) constellation[v] = qam_symbol(desc->modulation_order, (uint32_t)v);
  // What the transmitter places at FFT bin b of word w: data element k (>= 0),
  // reference element r (encoded ~r), or nothing.
  std::vector<int32_t> bin_code((size_t)W * N, INT32_MIN);
  for (int w = 0; w < W; ++w)
    for (int c = 0; c < C; ++c) {
      const int8_t k = f->h_kind[(size_t)w * C + c];
      const int32_t idx = f->h_index[(size_t)w * C + c];
      if (k == HPX_RE_DATA) bin_code[(size_t)w * N + f->h_bins[c]] = idx;
      else if (k == HPX_RE_REFERENCE) bin_code[(size_t)w * N + f->h_bins[c]] = ~idx;
    }

  // Transmitter descriptors (see hpx_frame): the staged bits of word w start at Philox
  // block (k0 m) / 128, so data element k sits at bit (k - k0) m + (k0 m) mod 128.
  if (nr >= (1 << 24)) {
    release(f);
    return hpx_fail(HPX_ERR_ARG, "frame: too many reference elements");
  }
  std::vector<int32_t> tx_src((size_t)W * N, -1), tx_regular(W, 0), tx_bitoff(W, 0);
  const int comb = desc->pilot_comb;
  for (int w = 0; w < W; ++w) {
    const int64_t k0 = f->h_data_offset[w];
    const int32_t off0 = (int32_t)((k0 * m) & 127);
    bool regular = true;
    for (int c = 0; c < C; ++c) {
      const int8_t k = f->h_kind[(size_t)w * C + c];
      const int32_t idx = f->h_index[(size_t)w * C + c];
      int32_t& dst = tx_src[(size_t)w * N + f->h_bins[c]];
      if (k == HPX_RE_DATA) {
        dst = (int32_t)((idx - k0) * m) + off0;
        regular = regular && idx == k0 + c;
      } else {
        regular = false;
        if (k == HPX_RE_REFERENCE) dst = -2 - ((idx << 6) | (comb > 1 ? c % comb : 0));
      }
    }
    tx_regular[w] = regular ? 1 : 0;
    tx_bitoff[w] = off0;
  }
  std::vector<float2> constellation_lsb(desc->modulation_order);
  for (int raw = 0; raw < desc->modulation_order; ++raw) {
    uint32_t v = 0;
    for (int i = 0; i < m; ++i) v |= (((uint32_t)raw >> i) & 1u) << (m - 1 - i);
    constellation_lsb[raw] = constellation[v];
  }

  hpx_status s = HPX_OK;
  if ((s = upload(&f->d_prefix, f->h_prefix)) != HPX_OK ||
      (s = upload(&f->d_zero_prefix, f->h_zero_prefix)) != HPX_OK ||
      (s = upload(&f->d_word_start, f->h_word_start)) != HPX_OK ||
      (s = upload(&f->d_window_start, f->h_window_start)) != HPX_OK ||
      (s = upload(&f->d_data_offset, f->h_data_offset)) != HPX_OK ||
      (s = upload(&f->d_num_data_word, num_data_word)) != HPX_OK ||
      (s = upload(&f->d_kind, f->h_kind)) != HPX_OK || (s = upload(&f->d_index, f->h_index)) != HPX_OK ||
      (s = upload(&f->d_bins, f->h_bins)) != HPX_OK || (s = upload(&f->d_data_column, data_column)) != HPX_OK ||
      (s = upload(&f->d_data_word, data_word)) != HPX_OK || (s = upload(&f->d_twiddle, tw)) != HPX_OK || (s = upload(&f->d_stage_twiddle, stw)) != HPX_OK ||
      (s = upload(&f->d_pilots, pilots)) != HPX_OK || (s = upload(&f->d_bin_code, bin_code)) != HPX_OK ||
      (s = upload(&f->d_constellation, constellation)) != HPX_OK || (s = upload(&f->d_tx_src, tx_src)) != HPX_OK ||
      (s = upload(&f->d_tx_regular, tx_regular)) != HPX_OK || (s = upload(&f->d_tx_bitoff, tx_bitoff)) != HPX_OK ||
      (s = upload(&f->d_constellation_lsb, constellation_lsb)) != HPX_OK) {
    release(f);
    return s;
  }
  *out = f;
  return HPX_OK;
}

hpx_status hpx_frame_destroy(hpx_frame* frame) {
  release(frame);
  return HPX_OK;
}

hpx_status hpx_frame_get_info(const hpx_frame* frame, hpx_frame_info* info) {
  if (!frame || !info) return hpx_fail(HPX_ERR_ARG, "frame_info: null argument");
  *info = frame->info;
  return HPX_OK;
}

}  // extern "C"
