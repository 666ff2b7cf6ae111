// The batched drop pipeline: realize -> transmit -> propagate + AWGN ->
// demodulate -> estimate / equalize / demap / count, all stream-ordered.
#include "hpx_internal.cuh"

struct hpx_ls;

struct hpx_link {
  const hpx_frame* frame;
  const hpx_fading* fading;
  const hpx_ls* ls;
  int estimator, equalizer, max_drops;
  int T, D, C, W;
  void* state = nullptr;  // fading state [max_drops]
  hpx_cf32* x = nullptr;  // [max_drops][ntx][T]
  hpx_cf32* y = nullptr;  // [max_drops][nrx][T + D]
  hpx_cf32* grid = nullptr;  // [max_drops][nrx][W][C]
};

static void link_release(hpx_link* l) {
  if (!l) return;
  if (l->state) cudaFree(l->state);
  if (l->x) cudaFree(l->x);
  if (l->y) cudaFree(l->y);
  if (l->grid) cudaFree(l->grid);
  delete l;
}

// Workspace bytes per drop of a link (fading state, transmit and receive
// samples, received grid).
static size_t link_bytes_per_drop(const hpx_frame* fr, const hpx_fading* f) {
  const size_t T = fr->info.samples_per_frame, D = f->max_delay, C = fr->info.num_columns, W = fr->info.num_words;
  return f->stride + sizeof(hpx_cf32) * (f->ntx * T + f->nrx * (T + D) + f->nrx * W * C);
}

extern "C" {

hpx_status hpx_link_workspace_bytes(const hpx_frame* frame, const hpx_fading* fading, int32_t num_drops, int64_t* bytes) {
  if (!frame || !fading || !bytes || num_drops < 0) return hpx_fail(HPX_ERR_ARG, "link_workspace: bad argument");
  *bytes = (int64_t)link_bytes_per_drop(frame, fading) * num_drops;
  return HPX_OK;
}

hpx_status hpx_link_create(const hpx_frame* frame, const hpx_fading* fading, const hpx_ls* ls, int32_t estimator,
                           int32_t equalizer, int32_t max_drops, hpx_link** out) {
  if (!frame || !fading || !out) return hpx_fail(HPX_ERR_ARG, "link: null argument");
  *out = nullptr;
  if (estimator != HPX_EST_IDEAL && estimator != HPX_EST_LS) return hpx_fail(HPX_ERR_ARG, "link: unknown estimator");
  if (estimator == HPX_EST_LS && !ls) return hpx_fail(HPX_ERR_ARG, "link: LS estimation needs an hpx_ls table");
  if (estimator == HPX_EST_LS && (fading->nrx != 1 || fading->ntx != 1))
    return hpx_fail(HPX_ERR_UNSUPPORTED, "Least-Squares channel estimation is only implemented for SISO links");
  if (estimator == HPX_EST_LS && !hpx_ls_matches_frame(ls, frame))
    return hpx_fail(HPX_ERR_SHAPE, "link: the LS table was built for another frame layout");
  if (equalizer != HPX_EQ_ZF && equalizer != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "link: unknown equalizer");
  if (max_drops < 1 || max_drops > 65535) return hpx_fail(HPX_ERR_ARG, "link: max_drops must be in [1, 65535]");
  hpx_link* l = new hpx_link();
  l->frame = frame;
  l->fading = fading;
  l->ls = ls;
  l->estimator = estimator;
  l->equalizer = equalizer;
  l->max_drops = max_drops;
  l->T = frame->info.samples_per_frame;
  l->D = fading->max_delay;
  l->C = frame->info.num_columns;
  l->W = frame->info.num_words;
  const size_t B = max_drops;
  cudaError_t e;
  if ((e = cudaMalloc(&l->state, fading->stride * B)) != cudaSuccess ||
      (e = cudaMalloc(&l->x, sizeof(hpx_cf32) * B * fading->ntx * l->T)) != cudaSuccess ||
      (e = cudaMalloc(&l->y, sizeof(hpx_cf32) * B * fading->nrx * (size_t)(l->T + l->D))) != cudaSuccess ||
      (e = cudaMalloc(&l->grid, sizeof(hpx_cf32) * B * fading->nrx * (size_t)l->W * l->C)) != cudaSuccess) {
    link_release(l);
    return hpx_cuda_status(e, "link workspace");
  }
  *out = l;
  return HPX_OK;
}

hpx_status hpx_link_destroy(hpx_link* link) {
  link_release(link);
  return HPX_OK;
}

hpx_status hpx_link_run(const hpx_link* l, uint64_t seed, int64_t drop0, int32_t num_drops, const float* noise_power,
                        uint32_t* errors, void* stream) {
  if (!l || !errors) return hpx_fail(HPX_ERR_ARG, "link_run: null argument");
  if (num_drops < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "link_run: bad drop range");
  if (num_drops > l->max_drops) return hpx_fail(HPX_ERR_ARG, "link_run: %d drops exceed the workspace (%d)", num_drops,
                                                l->max_drops);
  if (l->equalizer == HPX_EQ_LMMSE && !noise_power) return hpx_fail(HPX_ERR_ARG, "link_run: LMMSE needs noise powers");
  if (num_drops == 0) return HPX_OK;
  const hpx_fading* f = l->fading;
  HPX_TRY(hpx_fading_realize(f, seed, drop0, num_drops, l->state, stream));
  HPX_TRY(hpx_ofdm_modulate_bits(l->frame, seed, drop0, num_drops, f->ntx, l->x, stream));
  HPX_TRY(hpx_fading_propagate(f, l->state, num_drops, l->x, l->T, l->y, noise_power, seed, drop0, stream));
  HPX_TRY(hpx_ofdm_demodulate(l->frame, l->y, l->T + l->D, num_drops * f->nrx, l->C, l->grid, stream));
  if (l->estimator == HPX_EST_IDEAL)
    return hpx_detect_ideal(f, l->state, l->frame, l->equalizer, l->grid, l->C, noise_power, seed, drop0, num_drops,
                            errors, stream);
  return hpx_detect_ls(l->ls, l->equalizer, l->grid, l->C, noise_power, seed, drop0, num_drops, errors, stream);
}

}  // extern "C"
