// Batched drops for callers that cannot allocate device memory.
//
// hpx_link_run needs an hpx_link, whose workspace hpx_link_create obtains with
// cudaMalloc. Some callers cannot do that: a host application whose device memory
// is already fully reserved by its own pool allocator (cudaMalloc would fail or
// fragment that pool), latency-critical loops that must not pay cudaMalloc's
// implicit synchronization and unbounded latency after start-up, and plugins that
// are not allowed to own device allocations at all. hpx_link_run_static serves
// them from one fixed array in the library's own device image instead.
//
// The array is a file-scope __device__ variable of kStaticScratchBytes (64 MiB):
// every GPU that loads this library holds it until the process exits. Host code
// cannot use the array's name as a device address, so the first call on each
// device looks its address up with cudaGetSymbolAddress while that device is
// current and caches it. Under CUDA's lazy module loading that lookup is also when
// the device reserves the 64 MiB, so a caller whose pool allocator takes the rest
// of device memory makes this first call at start-up, before the pool grows (a call
// with num_drops = 0 does the set-up and nothing else), and before any stream
// capture. All calls on a device share the array and each call overwrites what it
// uses, so calls whose work overlaps on the GPU (different streams, or host threads
// without ordering) race and must be serialized by the caller.
#include <mutex>

#include "hpx_internal.cuh"

namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_link_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_address[kMaxDevices] = {};

size_t round_up(size_t v) { return (v + 255) / 256 * 256; }

// Device address of the scratch array on the current device (looked up once).
hpx_status scratch_address(void** out) {
  int dev = 0;
  HPX_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return hpx_fail(HPX_ERR_UNSUPPORTED, "link_run_static: device %d", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_address[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_link_scratch);
    if (e != cudaSuccess) return hpx_cuda_status(e, "cudaGetSymbolAddress(link scratch)");
    g_scratch_address[dev] = p;
  }
  *out = g_scratch_address[dev];
  return HPX_OK;
}

}  // namespace

extern "C" hpx_status hpx_link_run_static(const hpx_frame* frame, const hpx_fading* fading, const hpx_ls* ls,
                                          int32_t equalizer, uint64_t seed, int64_t drop0, int32_t num_drops,
                                          const float* noise_power, uint32_t* errors, void* stream) {
  if (!frame || !fading || !errors) return hpx_fail(HPX_ERR_ARG, "link_run_static: null argument");
  if (equalizer != HPX_EQ_ZF && equalizer != HPX_EQ_LMMSE)
    return hpx_fail(HPX_ERR_ARG, "link_run_static: unknown equalizer");
  if (equalizer == HPX_EQ_LMMSE && !noise_power) return hpx_fail(HPX_ERR_ARG, "link_run_static: LMMSE needs noise powers");
  if (ls && (fading->nrx != 1 || fading->ntx != 1))
    return hpx_fail(HPX_ERR_UNSUPPORTED, "Least-Squares channel estimation is only implemented for SISO links");
  // the LS receiver lays the grid out by its table's frame: it must be this frame's
  if (ls && !hpx_ls_matches_frame(ls, frame))
    return hpx_fail(HPX_ERR_SHAPE, "link_run_static: the LS table was built for another frame layout");
  if (num_drops < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "link_run_static: bad drop range");
  const size_t T = frame->info.samples_per_frame, D = fading->max_delay, C = frame->info.num_columns,
               W = frame->info.num_words;
  const size_t B = (size_t)num_drops;
  const size_t state_bytes = round_up(fading->stride * B);
  const size_t x_bytes = round_up(sizeof(hpx_cf32) * B * fading->ntx * T);
  const size_t y_bytes = round_up(sizeof(hpx_cf32) * B * fading->nrx * (T + D));
  const size_t grid_bytes = round_up(sizeof(hpx_cf32) * B * fading->nrx * W * C);
  const size_t per_drop = round_up(fading->stride) + sizeof(hpx_cf32) * (fading->ntx * T + fading->nrx * (T + D) +
                                                                        fading->nrx * W * C);
  if (state_bytes + x_bytes + y_bytes + grid_bytes > kStaticScratchBytes)
    return hpx_fail(HPX_ERR_ARG,
                    "link_run_static: %d drops need %zu bytes of scratch but the static array holds %zu bytes "
                    "(at most about %zu drops of this link per call)",
                    num_drops, state_bytes + x_bytes + y_bytes + grid_bytes, kStaticScratchBytes,
                    per_drop ? kStaticScratchBytes / per_drop : (size_t)0);
  void* base = nullptr;
  HPX_TRY(scratch_address(&base));  // also the set-up call: num_drops = 0 stops after it
  if (num_drops == 0) return HPX_OK;
  unsigned char* p = static_cast<unsigned char*>(base);
  void* state = p;
  hpx_cf32* x = reinterpret_cast<hpx_cf32*>(p + state_bytes);
  hpx_cf32* y = reinterpret_cast<hpx_cf32*>(p + state_bytes + x_bytes);
  hpx_cf32* grid = reinterpret_cast<hpx_cf32*>(p + state_bytes + x_bytes + y_bytes);
  // Every scratch buffer is written in full before it is read (state by the
  // realization, x by the transmitter, y by the propagation, grid by the
  // demodulator), so nothing carried over from an earlier call is used.
  HPX_TRY(hpx_fading_realize(fading, seed, drop0, num_drops, state, stream));
  HPX_TRY(hpx_ofdm_modulate_bits(frame, seed, drop0, num_drops, fading->ntx, x, stream));
  HPX_TRY(hpx_fading_propagate(fading, state, num_drops, x, (int32_t)T, y, noise_power, seed, drop0, stream));
  HPX_TRY(hpx_ofdm_demodulate(frame, y, (int64_t)(T + D), num_drops * fading->nrx, (int32_t)C, grid, stream));
  if (!ls)
    return hpx_detect_ideal(fading, state, frame, equalizer, grid, (int32_t)C, noise_power, seed, drop0, num_drops,
                            errors, stream);
  return hpx_detect_ls(ls, equalizer, grid, (int32_t)C, noise_power, seed, drop0, num_drops, errors, stream);
}
