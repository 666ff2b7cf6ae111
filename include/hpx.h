/*
 * hpx.h -- C ABI of the GB300 Monte Carlo link engine for HermesPy's OFDM
 * fading-link drop loop.
 *
 * Conventions
 *   - Complex samples are interleaved float32 pairs (hpx_cf32), i.e. the memory
 *     layout of numpy/torch complex64.
 *   - Every data pointer passed to a compute entry point is a DEVICE pointer on
 *     the current CUDA device; descriptors (hpx_frame_desc, hpx_fading_desc) hold
 *     HOST pointers and are copied at create time.
 *   - Batched buffers are dense, batch index outermost, shapes given in brackets.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream). Compute entry
 *     points only enqueue work; they never synchronize and never allocate.
 *     Handles (*_create) allocate their device tables once.
 *   - Every entry point returns an hpx_status; hpx_last_error() gives the
 *     message of the last failure on the calling thread. The Python layer maps
 *     HPX_ERR_ARG/HPX_ERR_SHAPE to ValueError, HPX_ERR_UNSUPPORTED to
 *     NotImplementedError and the rest to RuntimeError, as the reference does.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the HermesPy source tree).
 */
#ifndef HPX_H_
#define HPX_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float re, im; } hpx_cf32;

typedef enum {
  HPX_OK = 0,
  HPX_ERR_ARG = 1,         /* invalid argument          -> ValueError          */
  HPX_ERR_SHAPE = 2,       /* shape / size mismatch     -> ValueError          */
  HPX_ERR_UNSUPPORTED = 3, /* configuration not covered -> NotImplementedError */
  HPX_ERR_CUDA = 4,        /* CUDA runtime failure      -> RuntimeError        */
  HPX_ERR_NUMERIC = 5,     /* numerical failure         -> RuntimeError        */
  HPX_ERR_TIMEOUT = 6      /* bounded device wait ran out -> RuntimeError      */
} hpx_status;

/* Library version (major*10000 + minor*100 + patch). */
int hpx_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* hpx_last_error(void);

/* ----------------------------------------------------------- device status
 * Failures found on the device reach the caller in two ways, replacing the
 * reference's per-sample exception path (core/pymonte/actors.py:444-452, where a
 * failing drop raises into the actor and the campaign stops):
 *   - per drop: the bit-error word of every detection entry point (hpx_link_run,
 *     hpx_detect_*, hpx_uneven_run, ...) carries flag bits; a drop whose word has
 *     one of them holds no valid count;
 *   - per handle: handles whose kernels wait on the tensor cores or on TMA
 *     (hpx_lmmse, hpx_cnn) keep a sticky status word that their entry points set
 *     when a bounded wait runs out (~20 ms); later launches on the handle then skip
 *     their work and flag their drops, until hpx_*_status clears the word. */
#define HPX_DROP_TIMEOUT 0x80000000u /* a bounded tensor-core / TMA wait ran out */
#define HPX_DROP_NUMERIC 0x40000000u /* NaN / inf noise power, or a non-finite equalizer pivot */
#define HPX_DROP_COUNT 0x3fffffffu   /* mask of the bit-error count */

/* HPX_OK if no word of a HOST copy of per-drop error words carries a flag, else
 * HPX_ERR_TIMEOUT or HPX_ERR_NUMERIC (timeouts first) with the first flagged
 * drop's index in hpx_last_error(). */
hpx_status hpx_drop_status(const uint32_t* errors, int64_t num_drops);

/* ------------------------------------------------------------------ frames */

/* Element types of the resource grid, as ElementType
 * (modem/waveforms/orthogonal/waveform.py:39-49). */
enum { HPX_RE_REFERENCE = 0, HPX_RE_DATA = 1, HPX_RE_NULL = 2 };

typedef struct {
  int32_t num_subcarriers;   /* N, power of two in [64, 4096] (FFT size, oversampling 1) */
  int32_t num_words;         /* OFDM symbols per frame */
  int32_t num_columns;       /* grid columns described by `kind` (<= N) */
  int32_t modulation_order;  /* 2, 4, 16, 64 or 256 */
  int32_t dc_suppression;    /* 1: roll the upper half of the grid past DC (ofdm.py:116-120) */
  const int32_t* prefix;     /* [num_words] prefix length in samples */
  const int32_t* zero_prefix;/* [num_words] 1 = zero padding, 0 = cyclic prefix (may be NULL) */
  const int8_t* kind;        /* [num_words * num_columns] HPX_RE_* per resource element */
  int32_t pilot_comb;        /* 0 or 1: every stream sends every reference element (the reference's
                              * behaviour); P > 1: stream s sends the reference element of grid
                              * column c only if c % P == s % P and zero otherwise (per-stream
                              * pilots for MIMO estimation; no counterpart in the reference) */
} hpx_frame_desc;

typedef struct hpx_frame hpx_frame;

typedef struct {
  int32_t num_subcarriers, num_words, num_columns, modulation_order, bits_per_symbol;
  int32_t num_data;          /* data elements per frame and stream */
  int32_t num_refs;          /* reference elements per frame and stream */
  int32_t samples_per_frame; /* T */
} hpx_frame_info;

/* Build the device tables of one frame layout: the grid bookkeeping of
 * OrthogonalWaveform (resource_mask, samples_per_frame, pilot_symbols;
 * modem/waveforms/orthogonal/waveform.py:1140-1211, modem/waveform.py:797-820). */
hpx_status hpx_frame_create(const hpx_frame_desc* desc, hpx_frame** out);
hpx_status hpx_frame_destroy(hpx_frame* frame);
hpx_status hpx_frame_get_info(const hpx_frame* frame, hpx_frame_info* info);

/* ------------------------------------------------------- bits and mapping */

/* Data bits of `num_streams` streams of drops [drop0, drop0+num_drops), one byte
 * (0/1) per bit: bits[num_drops][num_streams][bits_per_stream].
 * Replaces RandomBitsSource.generate_bits (modem/bits_source.py:62-63) with the
 * engine's Philox4x32-10 stream (domain 1). */
hpx_status hpx_bits_generate(uint64_t seed, int64_t drop0, int32_t num_drops, int32_t num_streams,
                             int64_t bits_per_stream, uint8_t* bits, void* stream);

/* Gray PSK/QAM mapping, MSB first: bits[num_symbols * log2(order)] -> symbols.
 * Replaces PskQamMapping.get_symbols (modem/tools/psk_qam_mapping.py:104-169). */
hpx_status hpx_qam_map(int32_t order, const uint8_t* bits, int64_t num_symbols, hpx_cf32* symbols,
                       void* stream);

/* Hard demapping, bit-exact with PskQamMapping.detect_bits
 * (modem/tools/psk_qam_mapping.py:171-259) evaluated in float64 on the same
 * (float32) symbols: ties and NaN give 0. */
hpx_status hpx_qam_demap(int32_t order, const hpx_cf32* symbols, int64_t num_symbols, uint8_t* bits,
                         void* stream);

/* Bit errors of `batch` pairs of 0/1 byte vectors a[batch][len_a], b[batch][len_b]
 * after zero-padding the shorter one: errors[batch].
 * Replaces BitErrorEvaluator.evaluate (modem/evaluators.py:239-258). */
hpx_status hpx_count_errors(const uint8_t* a, int64_t len_a, const uint8_t* b, int64_t len_b,
                            int32_t batch, uint64_t* errors, void* stream);

/* -------------------------------------------------------------------- OFDM */

/* Place + modulate: data[batch][num_data] -> samples[batch][T].
 * Replaces OrthogonalWaveform.place + modulate with OFDMWaveform._forward_transformation
 * (modem/waveforms/orthogonal/waveform.py:1221-1258, 1292-1323; ofdm.py:98-130). */
hpx_status hpx_ofdm_modulate(const hpx_frame* frame, const hpx_cf32* data, int32_t batch,
                             hpx_cf32* samples, void* stream);

/* Modulate an already placed grid: grid[batch][num_words][grid_columns] (columns
 * 0..grid_columns-1 of the reference's (words, N) grid) -> samples[batch][T].
 * Replaces OrthogonalWaveform.modulate on the output of place
 * (modem/waveforms/orthogonal/waveform.py:1292-1323; ofdm.py:98-130). */
hpx_status hpx_ofdm_modulate_grid(const hpx_frame* frame, const hpx_cf32* grid, int32_t grid_columns, int32_t batch,
                                  hpx_cf32* samples, void* stream);

/* Fused bits -> map -> place -> modulate for the engine's Philox bits:
 * samples[num_drops][num_streams][T]. Replaces TransmittingModemBase._transmit's
 * bit generation, __map and __modulate (modem/modem.py:747-888). */
hpx_status hpx_ofdm_modulate_bits(const hpx_frame* frame, uint64_t seed, int64_t drop0,
                                  int32_t num_drops, int32_t num_streams, hpx_cf32* samples,
                                  void* stream);

/* Demodulate: samples[batch][sample_stride] (first T used) -> grid[batch][num_words][num_columns],
 * columns 0..num_columns-1 of the reference's (words, N) grid.
 * Replaces OrthogonalWaveform.demodulate with OFDMWaveform._backward_transformation
 * (modem/waveforms/orthogonal/waveform.py:1325-1364; ofdm.py:133-161). */
hpx_status hpx_ofdm_demodulate(const hpx_frame* frame, const hpx_cf32* samples, int64_t sample_stride,
                               int32_t batch, int32_t num_columns, hpx_cf32* grid, void* stream);

/* Gather the data elements: grid[batch][num_words][grid_columns] -> out[batch][num_data].
 * Replaces OrthogonalWaveform.pick (modem/waveforms/orthogonal/waveform.py:1260-1290). */
hpx_status hpx_ofdm_pick(const hpx_frame* frame, const hpx_cf32* grid, int32_t grid_columns,
                         int32_t batch, hpx_cf32* out, void* stream);

/* ------------------------------------------------------------------ fading */

typedef struct {
  int32_t num_taps;             /* L (delays sorted ascending by the caller) */
  int32_t num_sinusoids;        /* S >= 0 */
  int32_t num_rx, num_tx;       /* antennas */
  double sampling_rate;         /* Hz */
  double doppler_frequency;     /* NLOS Doppler, Hz */
  double los_doppler_frequency; /* LOS Doppler, Hz */
  double gain;                  /* linear power gain */
  const double* delays;         /* [L] seconds */
  const double* power_profile;  /* [L] linear */
  const double* rice_factors;   /* [L] linear, +inf for pure LOS */
  const double* rx_correlation; /* [num_rx*num_rx] interleaved complex, or NULL */
  const double* tx_correlation; /* [num_tx*num_tx] interleaved complex, or NULL */
  const double* los_gains;      /* [L] explicit LOS gains, or NULL to derive sqrt(K/(1+K)) */
  const double* nlos_gains;     /* [L] explicit NLOS gains, or NULL to derive sqrt(1/((1+K)S)) */
} hpx_fading_desc;

typedef struct hpx_fading hpx_fading;

/* Validate and precompute a MultipathFadingChannel configuration
 * (channel/fading/fading.py:606-754): gains sqrt(K/(1+K)), sqrt(1/((1+K)S)),
 * delays rint(tau*fs). Raises HPX_ERR_ARG for the reference's ValueErrors. */
hpx_status hpx_fading_create(const hpx_fading_desc* desc, hpx_fading** out);
hpx_status hpx_fading_destroy(hpx_fading* fading);
/* Bytes of the per-drop realization state buffer for `num_drops` drops. */
hpx_status hpx_fading_state_bytes(const hpx_fading* fading, int32_t num_drops, int64_t* bytes);
/* D = round(max delay * fs): propagated frames have T + D samples. */
hpx_status hpx_fading_max_delay(const hpx_fading* fading, int32_t* samples);

/* Realize drops [drop0, drop0+num_drops) from the engine's Philox stream (domain 2)
 * into `state`. Replaces MultipathFadingChannel._realize + MultipathFadingRealization._sample
 * (channel/fading/fading.py:468-515, 893-910; channel/consistent.py:431-432, 475-485). */
hpx_status hpx_fading_realize(const hpx_fading* fading, uint64_t seed, int64_t drop0, int32_t num_drops,
                              void* state, void* stream);

/* Load explicit sample parameters (device float64 arrays): los_angles[B][L],
 * nlos_angles[B][L][S], los_phases[B][L], nlos_phases[B][L][S], spatial[B][Nrx][Ntx]
 * (interleaved complex). Mirrors the MultipathFadingSample constructor
 * (channel/fading/fading.py:153-214). */
hpx_status hpx_fading_load(const hpx_fading* fading, int32_t num_drops, const double* los_angles,
                           const double* nlos_angles, const double* los_phases, const double* nlos_phases,
                           const double* spatial, void* state, void* stream);

/* The float64 uniforms of drops [drop0, drop0+num_drops) in the realization's draw
 * layout [spatial Nrx*Ntx][LOS angle L][NLOS angles L*S][LOS phase L][NLOS phases L*S]:
 * uniforms[num_drops][num_draws]. Exposes what hpx_fading_realize consumes (the
 * reference's ConsistentUniform samples, channel/consistent.py:475-485). */
hpx_status hpx_fading_draws(const hpx_fading* fading, uint64_t seed, int64_t drop0, int32_t num_drops,
                            double* uniforms, void* stream);

/* Tap coefficients taps[B][L][num_samples] by direct sum of sinusoids.
 * Replaces MultipathFadingSample.__path_impulse_generator (channel/fading/fading.py:293-343). */
hpx_status hpx_fading_taps(const hpx_fading* fading, const void* state, int32_t num_drops,
                           int32_t num_samples, hpx_cf32* taps, void* stream);

/* Impulse-response CSI csi[B][Nrx][Ntx][num_samples][num_taps_out], num_taps_out =
 * min(1 + D, max_num_taps). Replaces MultipathFadingSample.state (fading.py:345-369). */
hpx_status hpx_fading_csi(const hpx_fading* fading, const void* state, int32_t num_drops,
                          int32_t num_samples, int32_t max_num_taps, hpx_cf32* csi, void* stream);

/* Propagate x[B][Ntx][num_samples] -> y[B][Nrx][num_samples + D] and, when
 * noise_power != NULL, add complex AWGN of power noise_power[b] from the engine's
 * Philox stream (domain 3, drop index drop0+b).
 * Replaces MultipathFadingSample._propagate (channel/fading/fading.py:371-406) and
 * AWGNRealization.add_to (simulation/rf/noise/model.py:143-160). */
hpx_status hpx_fading_propagate(const hpx_fading* fading, const void* state, int32_t num_drops,
                                const hpx_cf32* x, int32_t num_samples, hpx_cf32* y,
                                const float* noise_power, uint64_t seed, int64_t drop0, void* stream);

/* Ideal frequency-domain CSI H[B][Nrx][Ntx][num_words][num_columns] of a frame.
 * Replaces OFDMIdealChannelEstimation.estimate_channel
 * (simulation/modem/channel_estimation.py:215-295). */
hpx_status hpx_fading_ideal_csi(const hpx_fading* fading, const void* state, int32_t num_drops,
                                const hpx_frame* frame, int32_t num_columns, hpx_cf32* csi, void* stream);

/* ------------------------------------------------- estimation / detection */

typedef struct hpx_ls hpx_ls;

/* Least-squares interpolator of a SISO frame as a CSR map from the reference
 * elements' LS values to grid[num_words][num_columns] (host arrays, row-major rows).
 * The map is the one OrthogonalLeastSquaresChannelEstimation.estimate_channel applies
 * (modem/waveforms/orthogonal/channel.py:29-66). */
hpx_status hpx_ls_create(const hpx_frame* frame, int32_t num_columns, const int32_t* indptr,
                         const int32_t* indices, const float* weights, hpx_ls** out);
hpx_status hpx_ls_destroy(hpx_ls* ls);
/* grid[B][num_words][grid_columns] -> H[B][num_words][num_columns]. */
hpx_status hpx_ls_estimate(const hpx_ls* ls, const hpx_cf32* grid, int32_t grid_columns, int32_t batch,
                           hpx_cf32* estimate, void* stream);

/* Least-squares interpolators of `num_streams` streams under a pilot comb: the CSR
 * map stacks one table of num_words*num_columns rows per stream, each built from
 * the stream's own reference elements like the SISO table (indices number the
 * frame's reference elements). The reference's estimator stops at one stream
 * (modem/waveforms/orthogonal/channel.py:32-35); this is its per-stream extension. */
hpx_status hpx_ls_create_streams(const hpx_frame* frame, int32_t num_columns, int32_t num_streams,
                                 const int32_t* indptr, const int32_t* indices, const float* weights,
                                 hpx_ls** out);
/* grid[B][Nrx][num_words][grid_columns] -> H[B][Nrx][num_streams][num_words][num_columns]. */
hpx_status hpx_ls_estimate_streams(const hpx_ls* ls, const hpx_cf32* grid, int32_t grid_columns,
                                   int32_t num_rx, int32_t batch, hpx_cf32* estimate, void* stream);

/* Tap-domain LMMSE channel estimator with the channel's statistics (delays, powers,
 * Doppler) known: weighted LS of the tap gains on each pilot word, per-tap LMMSE
 * over the words with the Jakes correlation of the sum-of-sinusoids taps, then
 * the tap DFT on every element. No counterpart in the reference. Tables are built
 * at create time for one frame and one fading configuration. */
typedef struct hpx_lmmse hpx_lmmse;
hpx_status hpx_lmmse_create(const hpx_frame* frame, const hpx_fading* fading, int32_t num_columns,
                            hpx_lmmse** out);
/* The same estimator with the statistics of `statistics` used as a prior in each
 * pilot word's tap estimate: (A^H A + ridge_noise diag(1 / P_u))^-1 A^H y instead of
 * the weighted LS, P_u the prior tap powers, and the per-tap noise of that estimate
 * in the LMMSE over words. With design statistics (a uniform profile over a delay
 * window, a design Doppler, the prior noise of a design SNR) this is the robust LMMSE
 * of Li, Cimini and Sollenberger (IEEE Trans. Commun. 46(7), 1998), which needs no
 * knowledge of the channel's taps; the plain LS step is ill-conditioned on such a
 * dense delay grid when the band is partly occupied. No counterpart in the
 * reference (engine extension); ridge_noise = 0 is hpx_lmmse_create. */
hpx_status hpx_lmmse_create_regularized(const hpx_frame* frame, const hpx_fading* statistics, int32_t num_columns,
                                        double ridge_noise, hpx_lmmse** out);
hpx_status hpx_lmmse_destroy(hpx_lmmse* lmmse);
/* grid[B][Nrx][num_words][grid_columns], noise_power[B] (per element) ->
 * H[B][Nrx][Ntx][num_words][num_columns]. */
hpx_status hpx_lmmse_estimate(const hpx_lmmse* lmmse, const hpx_cf32* grid, int32_t grid_columns,
                              int32_t num_rx, int32_t batch, const float* noise_power, hpx_cf32* estimate,
                              void* stream);

/* Fused receiver with the tap-domain LMMSE estimate: grid[B][Nrx][num_words][grid_columns]
 * -> per drop the tap gains of every pair and word (as hpx_lmmse_estimate) in on-chip
 * memory -> per data element the channel, equalization (ZF / LMMSE), hard demap and
 * bit-error count -> errors[B]. Antenna pairs: 1x1, 2x1, 2x2, 4x1, 4x2, 4x4. The CSI
 * grid never reaches HBM. No counterpart in the reference. */
/* Sticky device status of the handle: synchronizes `stream`, returns
 * HPX_ERR_TIMEOUT if a bounded tensor-core wait of hpx_detect_lmmse ran out since
 * the last clear (HPX_OK otherwise) and clears the word when `clear` != 0. */
hpx_status hpx_lmmse_status(hpx_lmmse* lmmse, int32_t clear, void* stream);
/* Host-side fault injection for tests of the error path: marks the handle as if a
 * wait had run out (stream-ordered write of the status word; nothing faults on the
 * device). Later hpx_detect_lmmse launches skip and flag every drop HPX_DROP_TIMEOUT. */
hpx_status hpx_lmmse_inject_timeout(hpx_lmmse* lmmse, void* stream);
hpx_status hpx_detect_lmmse(const hpx_lmmse* lmmse, int32_t num_rx, int32_t mode, const hpx_cf32* grid,
                            int32_t grid_columns, const float* noise_var, uint64_t seed, int64_t drop0,
                            int32_t num_drops, uint32_t* errors, void* stream);

/* Channel-estimate error over the frame's data elements, per drop:
 * err[b] = sum |est - truth|^2, power[b] = sum |truth|^2 over pairs x data elements,
 * est/truth[B][pairs][num_words][csi_columns]; NMSE = sum err / sum power. */
hpx_status hpx_csi_error(const hpx_frame* frame, const hpx_cf32* estimate, const hpx_cf32* truth,
                         int32_t csi_columns, int32_t pairs, int32_t batch, double* err, double* power,
                         void* stream);

enum { HPX_EQ_ZF = 0, HPX_EQ_LMMSE = 1 };

/* Per-element equalization: H[B][Nrx][Ntx][K], y[B][Nrx][K] -> x[B][Ntx][K].
 * HPX_EQ_ZF replaces ZeroForcingChannelEqualization.equalize_channel
 * (modem/waveform.py:235-250: y / sum_tx h for one receive stream, pinv(H) y otherwise);
 * HPX_EQ_LMMSE solves (H^H H + s2 I) x = H^H y by Cholesky (no reference counterpart),
 * s2 = noise_var[b]. */
hpx_status hpx_equalize(int32_t mode, int32_t num_rx, int32_t num_tx, int64_t num_elements, int32_t batch,
                        const hpx_cf32* channel, const hpx_cf32* received, const float* noise_var,
                        hpx_cf32* equalized, void* stream);

/* Fused receiver for drops with ideal CSI: grid[B][Nrx][num_words][grid_columns] ->
 * ideal CSI (as hpx_fading_ideal_csi) -> pick -> equalize (ZF or LMMSE) -> hard demap ->
 * compare with the regenerated Philox bits -> errors[B] (bit errors per drop).
 * Replaces the estimate/pick/equalize/unmap chain of ReceivingModemBase._receive
 * (modem/modem.py:1192-1267) and BitErrorEvaluator (modem/evaluators.py:239-258). */
hpx_status hpx_detect_ideal(const hpx_fading* fading, const void* state, const hpx_frame* frame,
                            int32_t mode, const hpx_cf32* grid, int32_t grid_columns,
                            const float* noise_var, uint64_t seed, int64_t drop0, int32_t num_drops,
                            uint32_t* errors, void* stream);

/* Fused receiver for a CSI grid from any estimator: grid[B][Nrx][num_words][grid_columns]
 * and csi[B][Nrx][Ntx][num_words][csi_columns] -> pick -> equalize (ZF or LMMSE) -> hard
 * demap -> compare with the regenerated Philox bits -> errors[B]. The same chain as
 * hpx_detect_ideal (modem/modem.py:1192-1267, modem/evaluators.py:239-258) with the
 * channel read instead of computed; serves the LS, LMMSE and learned estimators. */
hpx_status hpx_detect_csi(const hpx_frame* frame, int32_t num_rx, int32_t num_tx, int32_t mode,
                          const hpx_cf32* grid, int32_t grid_columns, const hpx_cf32* csi,
                          int32_t csi_columns, const float* noise_var, uint64_t seed, int64_t drop0,
                          int32_t num_drops, uint32_t* errors, void* stream);

/* Fused SISO receiver with LS estimation: grid[B][num_words][grid_columns] -> LS ->
 * pick -> ZF (or LMMSE) -> hard demap -> errors[B]. */
hpx_status hpx_detect_ls(const hpx_ls* ls, int32_t mode, const hpx_cf32* grid, int32_t grid_columns,
                         const float* noise_var, uint64_t seed, int64_t drop0, int32_t num_drops,
                         uint32_t* errors, void* stream);

/* ------------------------------------------------- learned estimator (CNN) */

/* Residual CNN that refines per-stream LS estimates of a 16-pair MIMO grid (4x4
 * antennas) into the full channel: 6 conv layers, 3x3 kernels, 32 channels
 * (16 pairs x re/im), ReLU between layers, output = LS + last layer. BF16 weights
 * and activations, FP32 accumulation on the tensor cores. No counterpart in the
 * reference. Parameters: weights [6][32 out][9 taps][32 in] then biases [6][32],
 * FP32 (hpx_cnn_num_params values); `params` NULL initialises them from `seed`. */
typedef struct hpx_cnn hpx_cnn;
int32_t hpx_cnn_num_params(void);
hpx_status hpx_cnn_create(int32_t num_words, int32_t num_columns, int32_t max_batch, const float* params,
                          uint64_t seed, hpx_cnn** out);
hpx_status hpx_cnn_destroy(hpx_cnn* cnn);
hpx_status hpx_cnn_get_params(const hpx_cnn* cnn, float* params);
/* Gradient sums of the last training step (host copy, same layout as the parameters). */
hpx_status hpx_cnn_get_grads(const hpx_cnn* cnn, float* grads);
/* In place: csi[B][16][num_words][csi_columns] (LS estimate) -> refined estimate. */
hpx_status hpx_cnn_refine(const hpx_cnn* cnn, hpx_cf32* csi, int32_t csi_columns, int32_t batch, void* stream);
/* Sticky device status of the network's tensor-core forward pass (as
 * hpx_lmmse_status): HPX_ERR_TIMEOUT if a TMA or MMA wait ran out, in which case
 * the refined estimates of that launch are NaN. */
hpx_status hpx_cnn_status(hpx_cnn* cnn, int32_t clear, void* stream);
/* Host-side fault injection (as hpx_lmmse_inject_timeout): later hpx_cnn_refine
 * launches skip their tiles and write NaN estimates. */
hpx_status hpx_cnn_inject_timeout(hpx_cnn* cnn, void* stream);
/* One Adam step on ls/truth[B][16][num_words][num_columns] (B <= max_batch), loss =
 * sum |out - truth|^2 written to the device double `loss` (may be NULL). */
hpx_status hpx_cnn_train_step(hpx_cnn* cnn, const hpx_cf32* ls, const hpx_cf32* truth, int32_t csi_columns,
                              int32_t batch, float learning_rate, double* loss, void* stream);

/* Fused massive-MIMO receiver with ideal CSI (16 transmit streams, 16/32/64 receive
 * antennas): per data element the Gram H^H H and matched filter H^H y on the BF16
 * tensor cores with split (3-term) products and FP32 accumulation, FP32 Cholesky
 * (LMMSE: + s2 I; ZF: none), FP64 re-factorization for elements whose condition
 * estimate (max/min Cholesky pivot)^2 exceeds 1e6, hard demap, error count.
 * errors[B]; fp64_count[B] (may be NULL) = elements solved in FP64; equalized
 * (may be NULL) = x[B][16][num_data]. No counterpart in the reference. */
hpx_status hpx_detect_massive(const hpx_fading* fading, const void* state, const hpx_frame* frame,
                              int32_t mode, const hpx_cf32* grid, int32_t grid_columns,
                              const float* noise_var, uint64_t seed, int64_t drop0, int32_t num_drops,
                              uint32_t* errors, uint32_t* fp64_count, hpx_cf32* equalized, void* stream);

/* ------------------------------------------------------------------- noise */

/* Add complex AWGN of power noise_power[b] to samples[batch][num_streams][num_samples]
 * in place, from the engine's Philox stream (domain 3, drop drop0+b, stream id =
 * stream index). Replaces AWGN.realize + AWGNRealization.add_to
 * (simulation/rf/noise/model.py:143-178). */
hpx_status hpx_awgn_add(hpx_cf32* samples, int32_t batch, int32_t num_streams, int64_t num_samples,
                        const float* noise_power, uint64_t seed, int64_t drop0, void* stream);

/* ----------------------------------------------------------- synchronization */

/* Schmidl-Cox delay metric of `batch` received signals [batch][num_streams][num_samples]:
 * metric[b][0] = 0 and metric[b][1 + d] = sum_s |sum_{k<L/2} conj(x[d+k]) x[d+k+L/2]| for
 * d = 0 .. num_samples - L (L = symbol_length), i.e. num_samples - L + 2 doubles per
 * signal, the layout of SchmidlCoxSynchronization.synchronize's delay_powers
 * (modem/waveforms/orthogonal/ofdm.py:236-248). The caller's find_peaks and the -1
 * index correction (:250-255) follow on the host. Signals shorter than L write nothing. */
hpx_status hpx_sync_schmidl_cox(const hpx_cf32* signal, int32_t batch, int32_t num_streams, int64_t num_samples,
                                int32_t symbol_length, double* metric, void* stream);
/* Pilot correlation profile correlation[b][k] = sum_s |sum_j x[k - (P-1) + j] conj(pilot[j])|,
 * k = 0 .. num_samples + P - 2 (scipy.signal.correlate(x, pilot, "full") magnitudes summed
 * over streams), before the normalization and peak search of
 * CorrelationSynchronization.synchronize (modem/waveform_correlation_synchronization.py:119-170). */
hpx_status hpx_sync_correlation(const hpx_cf32* signal, int32_t batch, int32_t num_streams, int64_t num_samples,
                                const hpx_cf32* pilot, int32_t pilot_length, double* correlation, void* stream);

/* Frame starts from `batch` metrics of `length` doubles (either output above), the
 * peak search of scipy.signal.find_peaks(x, height, distance) as the two routines
 * call it: local maxima (plateau midpoints), height >= height * max(x) (or, with
 * normalize, x / max(x) >= height), then distance suppression by decreasing height.
 * Kept peaks in index order, plus `offset` (Schmidl-Cox: -1; correlation: 1 - P),
 * optionally clipped (negative -> 0, above clip_max -> clip_value) go to
 * starts[b][0 .. max_frames); counts[b] = number kept, -1 if more than 512 peaks
 * passed the height test. */
hpx_status hpx_sync_peaks(const double* metric, int32_t batch, int64_t length, int32_t normalize, double height,
                          int64_t distance, int64_t offset, int32_t clip, int64_t clip_max, int64_t clip_value,
                          int32_t max_frames, int64_t* starts, int32_t* counts, void* stream);

/* --------------------------------------------------------------------- FEC */

/* LDPC block code from the edges of its parity-check matrix H (edge e joins variable
 * edge_var[e] < N and check edge_chk[e] < M). Replaces the aff3ct LDPC wrapper of the
 * reference (fec/aff3ct/ldpc.cpp: LDPC::LDPC, encode, decode; fec/aff3ct_wrappers.py
 * LDPCCoding), whose H comes from an alist file: the encoder is systematic from the
 * reduced row-echelon form of H (K = N - rank(H) data bits at the non-pivot columns),
 * the decoder belief propagation with the flooding schedule and the sum-product check
 * update. */
typedef struct hpx_ldpc hpx_ldpc;
hpx_status hpx_ldpc_create(int32_t N, int32_t M, int32_t E, const int32_t* edge_var, const int32_t* edge_chk,
                           hpx_ldpc** out);
hpx_status hpx_ldpc_destroy(hpx_ldpc* code);
/* K, N and (host array of K, may be NULL) the codeword position of each data bit. */
hpx_status hpx_ldpc_info(const hpx_ldpc* code, int32_t* data_bits, int32_t* code_bits, int32_t* info_positions);
/* data[B][K] bits (one per byte) -> code[B][N] bits (LDPC::encode). */
hpx_status hpx_ldpc_encode(const hpx_ldpc* code, const uint8_t* data, int32_t B, uint8_t* out, void* stream);
/* Hard code bits hard[B][N] (LDPC::decode's hard input: bit b -> channel LLR 4 (1 - 2b)) or,
 * if hard is NULL, channel LLRs llr[B][N] (log P(0) / P(1)) -> data[B][K]. At most
 * `iterations` flooding iterations; with syndrome_checking the decoder stops once every
 * parity check holds and min_iterations have run. iterations_used[B] may be NULL. */
hpx_status hpx_ldpc_decode(const hpx_ldpc* code, const uint8_t* hard, const float* llr, int32_t B, int32_t iterations,
                           int32_t syndrome_checking, int32_t min_iterations, uint8_t* data, int32_t* iterations_used,
                           void* stream);

/* ------------------------------------------------------- batched drop loop */

enum { HPX_EST_IDEAL = 0, HPX_EST_LS = 1 };

typedef struct hpx_link hpx_link;

/* Device workspace of a link for `num_drops` drops per run (bytes). */
hpx_status hpx_link_workspace_bytes(const hpx_frame* frame, const hpx_fading* fading, int32_t num_drops,
                                    int64_t* bytes);
/* A simplex OFDM link over a fading channel with its workspace for up to
 * max_drops drops per run; `ls` is required for HPX_EST_LS (SISO only). */
hpx_status hpx_link_create(const hpx_frame* frame, const hpx_fading* fading, const hpx_ls* ls, int32_t estimator,
                           int32_t equalizer, int32_t max_drops, hpx_link** out);
hpx_status hpx_link_destroy(hpx_link* link);
/* Simulate drops [drop0, drop0+num_drops): realize, transmit Philox bits, propagate
 * with AWGN of power noise_power[b], demodulate, estimate, equalize, demap and
 * count bit errors into errors[num_drops]. Replaces one SimulationScenario._drop
 * (simulation/scenario.py:772-804) plus BitErrorEvaluator per drop. */
hpx_status hpx_link_run(const hpx_link* link, uint64_t seed, int64_t drop0, int32_t num_drops,
                        const float* noise_power, uint32_t* errors, void* stream);

/* The batched drop loop of hpx_link_run for callers that cannot allocate device
 * memory (a host whose device memory is reserved by its own pool allocator,
 * latency-critical loops that must not call cudaMalloc after start-up, plugins
 * that may not own device allocations). No counterpart in the reference: it is an
 * allocation-free variant of this library's own hpx_link_run. Its scratch is one
 * fixed 64 MiB array in the library's device image, held by every GPU that loads
 * the library until the process exits; the largest batch is what fits in it
 * (about 50 drops of the 4x4, 1024-subcarrier link), larger batches fail with
 * HPX_ERR_ARG and a message giving the limit. `ls` selects LS estimation (SISO,
 * table built on this frame's layout, else HPX_ERR_SHAPE); NULL selects ideal CSI.
 * The first call on a device looks up the array's device address; under CUDA's lazy
 * module loading that is also when the device reserves the 64 MiB, so make it at
 * start-up, before a pool allocator of the host takes the remaining device memory,
 * and before any stream capture (a call with num_drops = 0 does this set-up and
 * nothing else). Calls share the array: calls that overlap on the GPU race. Never
 * calls cudaMalloc or cudaFree. */
hpx_status hpx_link_run_static(const hpx_frame* frame, const hpx_fading* fading, const hpx_ls* ls,
                               int32_t equalizer, uint64_t seed, int64_t drop0, int32_t num_drops,
                               const float* noise_power, uint32_t* errors, void* stream);

/* --------------------------------------------------------- uneven batches */

/* One drop of an uneven batch. Frame: fft_size N in [128, 2048], floor(0.586 N)
 * used data subcarriers, cyclic prefix N*72/1024, DC suppression, num_words data
 * words, ideal CSI + LMMSE. Channel: num_taps Rayleigh taps k * tap_spacing apart
 * with power 10^(-tap_decay_db k / 10), sampled at N * subcarrier_spacing. */
typedef struct {
  int32_t num_rx, num_tx;    /* 1, 2, 4 or 8 */
  int32_t fft_size;
  int32_t num_words;
  int32_t modulation_order;  /* 4, 16, 64 or 256 */
  int32_t num_taps;          /* 1 .. 64 */
  double tap_decay_db;
  double doppler_frequency;  /* Hz */
} hpx_uneven_drop;

/* Drops of different antenna counts, FFT sizes, frame lengths, modulation orders,
 * channels and SNRs in ONE persistent launch: every CTA takes whole drops from an
 * atomic counter (longest first) and runs realize -> transmit -> propagate + AWGN
 * -> receive -> ideal CSI + LMMSE -> demap -> count with the homogeneous engine's
 * arithmetic, so each drop's errors equal those of hpx_link_run for that drop.
 * max_slots bounds the resident CTAs (one scratch slot each). No counterpart in the
 * reference (its Monte Carlo actors run drops one by one). */
typedef struct hpx_uneven hpx_uneven;
hpx_status hpx_uneven_create(const hpx_uneven_drop* drops, int32_t num_drops, double subcarrier_spacing,
                             double tap_spacing, int32_t num_sinusoids, int32_t max_slots, hpx_uneven** out);
hpx_status hpx_uneven_destroy(hpx_uneven* batch);
/* Data bits of every drop (host array [num_drops]). */
hpx_status hpx_uneven_bits(const hpx_uneven* batch, int64_t* bits_per_drop);
/* Launch shape: threads per CTA (128 or 256), CTAs per SM and kernel variant (0:
 * registers as needed, 1: capped for two 256-thread CTAs per SM, 2: capped for three,
 * only for batches whose drops have at most 4 antennas a side), picked by the caller's
 * autotuner. hpx_uneven_get_config reports the current shape and how many CTAs of
 * (threads, variant) fit one SM (0 for a variant the batch cannot use). */
hpx_status hpx_uneven_config(hpx_uneven* batch, int32_t threads, int32_t blocks_per_sm, int32_t variant);
hpx_status hpx_uneven_get_config(const hpx_uneven* batch, int32_t threads, int32_t variant, int32_t* cur_threads,
                                 int32_t* cur_blocks_per_sm, int32_t* cur_variant, int32_t* max_blocks_per_sm);
/* noise_power[num_drops], errors[num_drops] (drop d uses Philox drop index drop0 + d). */
hpx_status hpx_uneven_run(hpx_uneven* batch, uint64_t seed, int64_t drop0, const float* noise_power,
                          uint32_t* errors, void* stream);
/* Capture the launch (counter reset + persistent kernel) into a CUDA graph with these
 * arguments; hpx_uneven_replay launches it on `stream`. */
hpx_status hpx_uneven_capture(hpx_uneven* batch, uint64_t seed, int64_t drop0, const float* noise_power,
                              uint32_t* errors);
hpx_status hpx_uneven_replay(hpx_uneven* batch, void* stream);

/* ------------------------------------------------- Monte Carlo campaign */

/* Device-resident campaign over noise levels with the reference's confidence
 * stopping rule (core/pymonte/scalar.py:101-125): per level the sums of the
 * per-drop BER x and x^2 and the drop count stay on the GPU; a level stops once
 * 2 (1 - Phi(sqrt(n) accuracy / std)) < confidence (std > 0, n >= min_samples) or
 * it holds max_drops_per_level drops. Each batch assigns its drops round-robin to
 * the levels still active and runs them through hpx_link_run. Replaces the
 * actor/collector loop of core/pymonte/actors.py:23-253 for one link. */
typedef struct hpx_campaign hpx_campaign;
hpx_status hpx_campaign_create(int32_t num_levels, const float* noise_power, double accuracy, double confidence,
                               int32_t min_samples, int64_t max_drops_per_level, int32_t max_batch,
                               double bits_per_drop, hpx_campaign** out);
hpx_status hpx_campaign_destroy(hpx_campaign* campaign);
hpx_status hpx_campaign_reset(hpx_campaign* campaign);
/* Up to max_batches batches of `batch` drops (drop indices drop0, drop0+1, ...);
 * the host reads the number of active levels every `check_every` batches and
 * returns when none is left. Synchronizes `stream` at those checks. */
hpx_status hpx_campaign_run(hpx_campaign* campaign, hpx_link* link, uint64_t seed, int64_t drop0, int32_t batch,
                            int32_t max_batches, int32_t check_every, int64_t* drops_run,
                            int32_t* levels_active, void* stream);
/* The same loop for drop pipelines other than hpx_link_run (the staged MIMO
 * estimators: tap-domain LMMSE, per-stream LS, the learned estimator): per batch
 * the host enqueues hpx_campaign_assign (the noise power of each of the batch's
 * drops, dealt round-robin to the active levels, into noise_power[batch]), its own
 * pipeline on those powers, and hpx_campaign_accumulate (adds the drops' error
 * words to their levels and re-evaluates the stopping rule). hpx_campaign_poll
 * synchronizes `stream` and reads the number of active levels; it returns
 * HPX_ERR_TIMEOUT / HPX_ERR_NUMERIC if an accumulated drop carried a failure flag
 * (such drops stay out of the sums). None of the three allocates. */
hpx_status hpx_campaign_assign(hpx_campaign* campaign, int32_t batch, float* noise_power, void* stream);
hpx_status hpx_campaign_accumulate(hpx_campaign* campaign, int32_t batch, const uint32_t* errors, void* stream);
hpx_status hpx_campaign_poll(hpx_campaign* campaign, int32_t* levels_active, void* stream);
/* Host copies of the per-level drop counts, bit errors, BER sums and flags (any may be NULL). */
hpx_status hpx_campaign_results(const hpx_campaign* campaign, int64_t* drops, int64_t* errors,
                                double* ber_sum, double* ber_sq, int32_t* confident);

#ifdef __cplusplus
}
#endif

#endif /* HPX_H_ */
