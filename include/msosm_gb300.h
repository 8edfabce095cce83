/*
 * msosm_gb300.h -- C ABI of the GB300-native MS-OSM coherent-dedispersion engine.
 *
 * This is the drop-in boundary for the hot path of joezhouchenye/AcceleratedMS-OSM:
 * host code (the header-only C++ shim in include/compat/, or any FFI) calls these
 * functions; they drive hand-written sm_103a kernels on one GPU.  Plain pointers
 * and sizes only; no CUDA or torch types appear (streams are passed as void*,
 * meaning cudaStream_t, NULL = the legacy default stream).
 *
 * Every function returns an int status (MSOSM_OK = 0).  Nothing here calls
 * exit() or resets the device, unlike the reference's CUDA_CHECK / destructor
 * (gpu/include/gpu_common.cuh:42-62, dedispersion/msosm/msosm_gpu_batch.cpp:252-255).
 * msosm_last_error() returns the message of a handle's last failure.
 *
 * Threading: a handle is driven by one host thread at a time (the reference's
 * processor objects have the same rule).  All device work of a handle is ordered
 * on the stream passed to each call.
 */
#ifndef MSOSM_GB300_H
#define MSOSM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define MSOSM_OK 0
#define MSOSM_ERR_ARG 1         /* invalid argument */
#define MSOSM_ERR_STATE 2       /* call out of order (e.g. process before init) */
#define MSOSM_ERR_CUDA 3        /* a CUDA runtime call or kernel launch failed */
#define MSOSM_ERR_NOMEM 4       /* device or host allocation failed */
#define MSOSM_ERR_UNSUPPORTED 5 /* size/format outside what the engine supports */

/* ---- input sample formats (one complex sample per element) ----------------- */
#define MSOSM_IN_U16 0 /* uint16_pair, offset binary, 0 = no data (utils/include/globals.h:22-26) */
#define MSOSM_IN_C64 1 /* complex64 (float re, float im) */
#define MSOSM_IN_I8 2  /* int8 interleaved I/Q (psrdada NBIT=8) */

/* ---- output modes (bit flags) ----------------------------------------------- */
#define MSOSM_OUT_NONE 0 /* no series output (fold-only; needs an attached fold) */
#define MSOSM_OUT_C64 1  /* complex64 [D][B][M] -- the reference's fold-mode output_buffer_d */
#define MSOSM_OUT_U16 2  /* uint16_pair [D][B][M] -- the reference's stream-mode output */

typedef struct msosm_s msosm_t;
typedef struct msosm_fold_s msosm_fold_t;

/* Library version string and the text of a status code. */
const char *msosm_version(void);
const char *msosm_status_string(int status);

/* ---- host-only planning (no GPU needed) -------------------------------------
 * The reference's Prepare_MSOSM / Prepare_OSM public methods as free functions:
 * msosm_plan_nd        Nd per DM, Prepare_MSOSM ctor (msosm_prepare.cpp:25-46)
 * msosm_plan_min_order calculate_min_order (msosm_prepare.cpp:48-69): M_min
 * msosm_plan_segmentation segmentation(i) (msosm_prepare.cpp:215-284): 2M
 *                      per-bin block delays and the DM's delaycount
 * msosm_plan_response  generate_dedisp_params(i) (msosm_prepare.cpp:107-164):
 *                      2M complex64 (4M floats), FP64 inside
 * osm_plan             Prepare_OSM ctor + calculate_min_order (osm_prepare.cpp:3-28)
 */
int msosm_plan_nd(float bw, float f0, const float *dms, int num_dms, int *nd_out);
int msosm_plan_min_order(const int *nd, int num_dms, int *M_min_out);
int msosm_plan_segmentation(float bw, float f0, float dm, int nd, int M, int *delay_out, int *dc_out);
int msosm_plan_response(float bw, float f0, float dm, int M, float *H_out);
int osm_plan(float bw, float dm, float f0, unsigned long *nd_out, unsigned long *M_min_out);

/* ---- MS-OSM processor --------------------------------------------------------
 * msosm_create replaces Prepare_MSOSM(float bw, float *dm, float f0, int numDMs)
 *   (dedispersion/include/msosm_prepare.h:13, msosm_prepare.cpp:25-46) and the
 *   MSOSM_GPU_BATCH constructors (dedispersion/include/msosm_gpu_batch.h:16-17).
 *   bw = sampling rate = bandwidth in Hz, f0 = band bottom in Hz, dms copied.
 *   DMs must be ascending (the reference reads past its boundary table
 *   otherwise, msosm_prepare.cpp:239); DM 0 is an identity filter.
 * msosm_init replaces MSOSM_GPU_BATCH::initialize_uint16(int fftpoint, int batch,
 *   bool fold) (msosm_gpu_batch.h:19, msosm_gpu_batch.cpp:12-151): fftpoint 0
 *   picks 2*M_min, otherwise M = max(fftpoint/2, M_min).  in_format is an
 *   MSOSM_IN_* value, out_mode an MSOSM_OUT_* mask.  batch need not be a
 *   multiple of 4.  fftpoint must come out a power of two in [256, 2^24]; 2^23 and 2^24
 *   (long plain overlap-save filters) support MSOSM_OUT_C64 or MSOSM_OUT_U16 series
 *   output and the fused fold.
 */
int msosm_create(float bw, float f0, const float *dms, int num_dms, msosm_t **out);
int msosm_init(msosm_t *h, int fftpoint, int batch, int in_format, int out_mode);

/* ---- split precision ---------------------------------------------------------
 * No counterpart in the reference (its inverse transforms are cuFFT FP32,
 * msosm_gpu_batch.cpp:196-199,224-227).  MSOSM_PREC_FP32 (the default) runs the
 * FP32 register transform.  MSOSM_PREC_BF16X3 / MSOSM_PREC_FP16X3 run the inverse
 * transforms' 32-point DFT stages as tensor-core (tcgen05) contractions on 16-bit
 * operands split into hi + lo parts, three products per contraction (hi*hi +
 * lo*hi + hi*lo) accumulated in FP32; the chirp phase of the responses stays FP64
 * (msosm_plan_response) and every other step FP32.  FP16 operands are scaled by
 * powers of two from a running bound on the spectra, so they stay in range.
 * Available for fftpoint 2^18; MSOSM_ERR_UNSUPPORTED otherwise.  Call after
 * msosm_init; it may be changed between steps. */
#define MSOSM_PREC_FP32 0
#define MSOSM_PREC_BF16X3 1
#define MSOSM_PREC_FP16X3 2
int msosm_set_precision(msosm_t *h, int precision);
int msosm_get_precision(const msosm_t *h);

/* Geometry of the handle's last persistent inverse-transform launch (F >= 2^16):
 * CTAs, CTAs per SM the occupancy query reported, look-behind and intermediate
 * slots; zeros before the first such launch.  No counterpart in the reference. */
int msosm_get_launch_info(const msosm_t *h, int *grid, int *occupancy, int *lag, int *slots);

/* Return the L2 lines that persistent launches marked persisting (their access-policy
 * window over the intermediate slots) to normal and this context's persisting set-aside
 * to zero, e.g. before timing other GPU work in the same process; the next persistent
 * launch sets the set-aside again for its own slot ring (each launch sets it to the size
 * its ring needs).  Context state only, gone with the process.  No counterpart in the
 * reference. */
int msosm_reset_l2_persisting(void);

/* Planning results: M, M_min, F = 2M, batch, DM count, processor-wide delaycount
 * and the number of spectra kept in the ring (fft_block_size).  Any pointer may
 * be NULL.  Replaces the public members M, M_min, numDMs, delaycount of
 * Prepare_MSOSM (msosm_prepare.h:19-40) and fft_block_size (msosm_gpu_batch.h:54). */
int msosm_get_dims(const msosm_t *h, int *M, int *M_min, int *fftpoint, int *batch, int *num_dms,
                   int *delaycount, int *ring_blocks);
/* Nd_values (msosm_prepare.h:38), per-DM delaycount_values (:32). */
int msosm_get_nd(const msosm_t *h, int *nd_out);
int msosm_get_delaycounts(const msosm_t *h, int *dc_out);
/* delay_points[dm] (msosm_prepare.h:36): 2M ints. */
int msosm_get_delay_points(const msosm_t *h, int dm_index, int *out);
/* dedisp_params[dm] (msosm_prepare.h:34): 2M complex64 as 4M floats. */
int msosm_get_response(const msosm_t *h, int dm_index, float *out);

/* One streaming step: B*M new samples of the init'ed format from `in` (host or
 * device pointer; host memory should be pinned for an asynchronous copy), all
 * DMs dedispersed, outputs and the attached fold updated.  Asynchronous: a pinned
 * or device `in` must stay unchanged until the step is done (msosm_sync); a
 * pageable host `in` may be reused on return.  Host inputs are copied on the
 * handle's own stream, overlapping the previous step's transforms.  Replaces
 * MSOSM_GPU_BATCH::filter_block_uint16(uint16_pair*) (msosm_gpu_batch.h:20,
 * msosm_gpu_batch.cpp:178-236) and its complex64 / int8 variants.  A handle with
 * MSOSM_OUT_NONE and no fold attached runs only the forward transform: the step
 * advances the stream (tail, ring of spectra) and produces nothing. */
int msosm_process(msosm_t *h, const void *in, void *stream);
/* `nsteps` consecutive steps from one contiguous input of nsteps*B*M samples. */
int msosm_process_many(msosm_t *h, const void *in, int nsteps, void *stream);

/* ---- CUDA-graph capture ---------------------------------------------------------
 * No counterpart in the reference.  msosm_graph_create captures `nsteps` consecutive
 * steps of the handle reading `in` (device memory, nsteps*B*M samples at a fixed
 * address) into a CUDA graph: per step the forward passes, the one persistent inverse
 * launch and, with a fold attached, a device-side advance of the fold's phase.
 * msosm_graph_launch replays it on `stream` as the next nsteps steps (the caller
 * refills `in` between launches): the ring slots and the tail buffer repeat, so nsteps
 * must be a multiple of lcm(ring_blocks / B, 2), and the fold's time origin is set on
 * the device at each launch, so folding continues as with msosm_process.  Needs
 * fftpoint >= 65536, no writer and no kernel timing; the handle must not be
 * destroyed before its graphs.  Capture runs nothing and leaves the handle's state
 * as it was. */
typedef struct msosm_graph_s msosm_graph_t;
int msosm_graph_create(msosm_t *h, const void *in, int nsteps, msosm_graph_t **out);
int msosm_graph_launch(msosm_graph_t *g, void *stream);
int msosm_graph_destroy(msosm_graph_t *g);

/* Copy the last step's [D][B][M] output (format = the init'ed out_mode's series,
 * complex64 if both) to `out` (host or device).  Replaces
 * MSOSM_GPU_BATCH::get_output(uint16_pair*) (msosm_gpu_batch.h:21, .cpp:238-245). */
int msosm_get_output(msosm_t *h, void *out, void *stream);
/* Device pointer of the complex64 output, NULL unless MSOSM_OUT_C64.  Replaces
 * get_output_pointer() (msosm_gpu_batch.h:24). */
void *msosm_device_output(msosm_t *h);
/* Device pointer of the uint16_pair output, NULL unless MSOSM_OUT_U16. */
void *msosm_device_output_u16(msosm_t *h);
/* Number of steps processed so far. */
long long msosm_steps(const msosm_t *h);
/* cudaStreamSynchronize(stream) (synchronize(), msosm_gpu_batch.cpp:247-250, used
 * cudaDeviceSynchronize). */
int msosm_sync(msosm_t *h, void *stream);
/* Frees all device memory of the handle; never resets the device. */
int msosm_destroy(msosm_t *h);
const char *msosm_last_error(const msosm_t *h);

/* ---- kernel timing ------------------------------------------------------------
 * Takes the place of the reference's NVTX ranges "Convert and FFT", "Gather and
 * Multiply", "IFFT", "Discard and Convert" (msosm_gpu_batch.cpp:206-243) with
 * device-side numbers: when enabled, every kernel launch of the handle is
 * bracketed by CUDA events on its own stream.  msosm_profile_read (after the
 * stream is synchronised) returns, per kernel kind, the summed milliseconds,
 * the launches, how many of them were timed, and the F-point transforms done.
 * Launch and transform counts are kept even with timing off. */
#define MSOSM_KERNEL_FWD_PASS1 0 /* decode + forward column transforms */
#define MSOSM_KERNEL_FWD_PASS2 1 /* forward row transforms -> spectra ring */
#define MSOSM_KERNEL_INV_PASS1 2 /* delayed-bin gather x response + inverse column transforms */
#define MSOSM_KERNEL_INV_PASS2 3 /* inverse row transforms + discard/scale/encode/fold */
#define MSOSM_KERNEL_INV_FUSED 4 /* both inverse passes in one persistent launch (F >= 2^16) */
int msosm_profile_enable(msosm_t *h, int on);
int msosm_profile_reset(msosm_t *h);
int msosm_profile_read(msosm_t *h, int kind, double *ms_total, long long *launches, long long *timed,
                       long long *transforms);

/* ---- FFT-size autotuning ---------------------------------------------------------
 * No counterpart in the reference (it takes fftpoint from the command line or uses
 * 2*M_min).  Times fold-only processing of `steps` calls on this GPU for every
 * power-of-two fftpoint from max(min_fftpoint, 2*M_min) to max_fftpoint whose
 * buffers fit in free device memory, using at most 16 of the DMs (spread over the
 * list, the largest always included since it sets the ring), and returns the
 * fastest in samples x DM trials per second.  The caller caches the answer. */
int msosm_autotune(float bw, float f0, const float *dms, int num_dms, int batch, int in_format, int min_fftpoint,
                   int max_fftpoint, int steps, int *best_fftpoint, double *best_rate);

/* Launch shape of the persistent inverse transform: at most ctas_per_sm resident CTAs per
 * SM (0, the default, = as many as fit; fewer CTAs keep fewer intermediate slots in
 * flight, less L2 pressure at large F), and the transform order: DM trials in groups of
 * dm_group, window-major inside a group, so that consecutive transforms gather from
 * nearly the same spectra-ring lines (0 keeps the current order; 1 = DM-major; until set,
 * groups of 4 for transforms of up to 2^18 points and DM-major above).  Series outputs do
 * not depend on either; fused folds only to the order of their float sums.  No counterpart
 * in the reference. */
int msosm_set_launch_shape(msosm_t *h, int ctas_per_sm, int dm_group);
/* msosm_autotune over the FFT size, the windows per call (`batches`, num_batches
 * candidates) and the launch shape (as many CTAs per SM as fit, or one), fold-only on
 * at most 16 of the DMs; the fastest triple and its rate.  The radix plan and tile of
 * each size are fixed (one measured plan per size). */
int msosm_autotune_shape(float bw, float f0, const float *dms, int num_dms, int in_format, int min_fftpoint,
                         int max_fftpoint, const int *batches, int num_batches, int steps, int *best_fftpoint,
                         int *best_batch, int *best_ctas_per_sm, double *best_rate);

/* Failure-detection self-test (no counterpart in the reference): runs the persistent
 * transform's bounded device-side wait alone, on a counter preset to `preset` that
 * nothing else writes, waiting for `target` with a limit of timeout_ns (at most 2 s).
 * *timed_out = 1 when the wait ran out (the kernel raised its error flag and returned;
 * the context stays usable), *elapsed_ns = the wait's duration on %globaltimer. */
int msosm_selftest_wait(unsigned preset, unsigned target, unsigned long long timeout_ns, int *timed_out,
                        unsigned long long *elapsed_ns);

/* Tensor-core operand-layout self-test (no counterpart in the reference): one CTA
 * computes D[m][j] = sum_k A[m][k] * B[b_row0 + j][k] (m < 128, j < n, k < 64;
 * n = 32 or 64, b_row0 a multiple of 8) with tcgen05 MMAs from shared memory in
 * the layout the split-precision transform uses, FP32 accumulation in tensor
 * memory.  A (128 x 64) and B (64 x 64) are row-major 16-bit host arrays, FP16 or
 * (bf16 != 0) BF16; D is a host array of 128*n floats.  *timed_out = 1 when the
 * kernel's bounded wait for the MMAs ran out. */
int msosm_selftest_umma(int bf16, int n, int b_row0, const uint16_t *A, const uint16_t *B, float *D,
                        int *timed_out);

/* ---- per-DM output files -------------------------------------------------------
 * Replaces MSOSM_DataSave_Uring (data_save/include/msosm_data_save_uring.h:22-52,
 * msosm_data_save_uring.cpp:40-288) with pwrite worker threads (no liburing):
 * msosm_writer_create  config_save + initialize_uring: one file per DM,
 *                      <dir>/<prefix>_DM<value>.dat (decimals chosen as the reference
 *                      does), `slots` page-aligned host buffers of num_dms*bytes_per_dm
 *                      (pinned when a GPU is present); direct_io asks for O_DIRECT
 *                      (used when the file system accepts it)
 * msosm_attach_writer  after every msosm_process the handle's uint16 output (B*M
 *                      pairs per DM; the handle must have MSOSM_OUT_U16) is copied
 *                      into a free slot on the call's stream and written at offset
 *                      step*bytes_per_dm of each DM's file (copy_to_slot +
 *                      save_to_disk); blocks while every slot is busy
 * msosm_writer_write   the same from a host block [num_dms][bytes_per_dm]
 * msosm_writer_join    join_saving: wait for all writes; the first I/O or CUDA error */
typedef struct msosm_writer_s msosm_writer_t;
int msosm_writer_create(const char *dir, const char *prefix, const float *dms, int num_dms,
                        unsigned long long bytes_per_dm, int slots, int direct_io, msosm_writer_t **out);
int msosm_attach_writer(msosm_t *h, msosm_writer_t *w);
/* copy_to_slot (msosm_data_save_uring.cpp:100-110) for a handle without an attached
 * writer: the handle's last uint16 output into a free slot on `stream`, then written
 * by a worker at the next step offset; blocks while every slot is busy. */
int msosm_writer_copy_output(msosm_writer_t *w, msosm_t *h, void *stream);
int msosm_writer_write(msosm_writer_t *w, const void *host_block);
int msosm_writer_join(msosm_writer_t *w);
const char *msosm_writer_last_error(const msosm_writer_t *w);
int msosm_writer_filename(const msosm_writer_t *w, int dm_index, char *buf, size_t len);
int msosm_writer_destroy(msosm_writer_t *w);

/* ---- DM derivative ---------------------------------------------------------------
 * No counterpart in the reference.  With the segmentation (integer block delays)
 * held fixed, the dedispersed series depends on DM only through the response,
 * and the chirp phase is linear in DM, so dx/dDM is the same pipeline run with
 * dH/dDM in place of H.  For folded-profile sharpness S = sum_k P_k^2, with
 * P_k = sum|x|^2 / n_k:  dS/dDM = sum_k 2 P_k * (sum 2 Re(conj(x) dx/dDM)) / n_k.
 * msosm_plan_response_derivative  dH/dDM for one DM (2M complex64, FP64 inside)
 * msosm_use_response_derivative   replace a handle's responses by dH/dDM, so its
 *                                 outputs are dx/dDM for the same input
 * msosm_fold_accumulate_cross     fold 2 Re(conj(x) dx) (x, dx: device complex64,
 *                                 num_series*size samples), counting the samples
 *                                 where |x|^2 != 0, as the power fold counts them */
int msosm_plan_response_derivative(float bw, float f0, float dm, int M, float *H_out);
int msosm_use_response_derivative(msosm_t *h);
int msosm_fold_accumulate_cross(msosm_fold_t *f, const void *x, const void *dx, void *stream);

/* ---- checkpoint / resume -------------------------------------------------------
 * No counterpart in the reference (its stream state lives only in device memory,
 * msosm_gpu_batch.cpp:50-52, 113-125).  The state of a stream is the previous
 * call's last M samples, the ring of past spectra and the call counter; it does
 * not depend on the DM list, so it can be restored into any handle with the same
 * M, batch and ring size.  msosm_state_bytes gives the buffer size; save/load copy
 * through a host (or device) buffer and synchronise `stream`.  The fold's state
 * (double sums, counts, time origin) is saved separately. */
size_t msosm_state_bytes(const msosm_t *h);
int msosm_save_state(msosm_t *h, void *buf, size_t bytes, void *stream);
int msosm_load_state(msosm_t *h, const void *buf, size_t bytes, void *stream);
size_t msosm_fold_state_bytes(const msosm_fold_t *f);
int msosm_fold_save_state(msosm_fold_t *f, void *buf, size_t bytes, void *stream);
int msosm_fold_load_state(msosm_fold_t *f, const void *buf, size_t bytes, void *stream);

/* ---- plain overlap-save (single DM) -----------------------------------------
 * osm_create replaces Prepare_OSM(float bw, float dm, float f0) / OSM_GPU_BATCH
 * (dedispersion/include/prepare.h:10, osm_gpu_batch.h:10): the filter order is
 * M = 2*next_pow2(Nd) (osm_prepare.cpp:15-28) and every bin has delay 0, so the
 * same engine runs it.  msosm_init then mirrors OSM_GPU_BATCH::initialize_uint16
 * (osm_gpu_batch.cpp:19-92) and msosm_process its filter_block_uint16 (:94-123). */
int osm_create(float bw, float dm, float f0, msosm_t **out);

/* ---- folding -----------------------------------------------------------------
 * msosm_fold_create replaces Fold_GPU(float period, float fs, unsigned long size,
 *   string, unsigned long time_bin) (folding/include/fold_gpu.h:13,
 *   fold_gpu.cpp:4-25) for `num_series` independent series (one per DM; the
 *   reference folds one).  time_bin 0 means period*fs bins, like the reference's -1.
 * msosm_fold_accumulate replaces calculate_intensity(pol1[, pol2]) followed by
 *   fold_data_phase() (fold_gpu.cpp:27-54): pol1/pol2 are device complex64
 *   series of num_series*size samples; pol2 NULL gives |a|^2, otherwise
 *   sqrt(|a|^2+|b|^2) (gpu/gpu_kernel.cu:430-444); zero samples are skipped; the
 *   fold's time origin advances by size/fs per call.
 * msosm_fold_read replaces get_folded_data() (fold_gpu.cpp:56-60): folded mean
 *   per bin (float, [num_series][time_bin]) and optionally the raw double sums
 *   and counts.  Any output pointer may be NULL.
 * msosm_attach_fold makes every msosm_process fold |x|^2 of each DM's new output
 *   into row d inside the inverse transform (no series round trip through HBM).
 *   The fold must have num_series == num_dms and size == B*M.
 */
int msosm_fold_create(float period, float fs, unsigned long size, unsigned long time_bin, int num_series,
                      msosm_fold_t **out);
int msosm_fold_accumulate(msosm_fold_t *f, const void *pol1, const void *pol2, void *stream);
int msosm_fold_read(msosm_fold_t *f, float *folded, double *sums, unsigned long long *counts, void *stream);
int msosm_fold_reset(msosm_fold_t *f, void *stream);
int msosm_fold_dims(const msosm_fold_t *f, unsigned long *time_bin, int *num_series, unsigned long *size);
int msosm_fold_destroy(msosm_fold_t *f);
int msosm_attach_fold(msosm_t *h, msosm_fold_t *f);
/* 2-pol fused fold (replaces Fold_GPU::calculate_intensity(a, b) + fold_data_phase,
 * fold_gpu.cpp:27-60, for two processors of the same plan): `first` writes |a|^2 of
 * every output sample into a buffer the fold owns (num_series*size floats), and every
 * msosm_process of `second` folds sqrt(|a|^2 + |b|^2) of the same samples -- the
 * reference's 2-pol intensity (gpu_kernel.cu:430-436) -- with no complex series written.
 * Per step: msosm_process(first, pol_a) then msosm_process(second, pol_b) on one stream.
 * Both handles: same DMs, batch and fftpoint (>= 65536), MSOSM_OUT_NONE. f = NULL
 * detaches both. */
int msosm_attach_fold_pol2(msosm_t *first, msosm_t *second, msosm_fold_t *f);

/* Replace DM trial dm_index's response by a caller-supplied one: F complex64 bins
 * (2F interleaved floats, host or device) in the transform's natural bin order.
 * No counterpart in the reference (its responses come only from
 * generate_dedisp_params, msosm_prepare.cpp:107-164). */
int msosm_set_response(msosm_t *h, int dm_index, const float *H);

/* ---- simulated pulsar baseband ---------------------------------------------------
 * Replaces SimulatedComplexSignal (simulated_pulsar/include/simulated_complex_signal.h:7-55,
 * simulated_complex_signal.cpp) and AWGN (simulated_pulsar/include/AWGN.h:8-17,
 * AWGN.cpp:3-58), generated on the GPU:
 * msosm_sim_create     SimulatedComplexSignal(bw, dm, f0, period): Np = period*fs
 *                      samples per period, Nd as Prepare_OSM computes it (:16-30)
 * msosm_sim_set_pulse  MSOSM_SIM_TEST_PULSE: the generator's three-component test
 *                      profile times complex Gaussian noise, a new realisation every
 *                      period (generate_test_pulse, :44-72); MSOSM_SIM_GAUSSIAN: one
 *                      Gaussian component of FWHM duty*period at phase 0.5;
 *                      MSOSM_SIM_IMPULSES: two impulses of 32767 per period at Np/2
 *                      and Np/2 + 2 (generate_pulsar_signal, :563-571)
 * msosm_sim_set_noise  additive complex AWGN at per-sample SNR snr_db against the
 *                      emission's mean power (generate_pulsar_signal's add_noise, SNR)
 * msosm_sim_generate   the next n samples of the dispersed stream (causal dispersion
 *                      response applied by the engine's overlap-save transform, its
 *                      Nd-sample delay skipped, :347-442), times `scale`, encoded as
 *                      MSOSM_IN_C64 / MSOSM_IN_U16 (offset binary, 0 kept as "no data")
 *                      / MSOSM_IN_I8 into `out` (host: returns with the data there;
 *                      device: asynchronous on `stream`).  Consecutive calls continue
 *                      the stream; every sample depends only on the seed and its index.
 * msosm_sim_info       Np, Nd, mean emission power per sample, noise sigma per quadrature
 * msosm_awgn           AWGN::generateNoiseSamples: n complex samples (2n floats, host or
 *                      device) with independent N(mean, stddev^2) quadratures, samples
 *                      first .. first+n-1 of the seed's noise stream.
 * Dispersion smear is limited to Nd < 2^23 samples (filter transform <= 2^24 points). */
#define MSOSM_SIM_TEST_PULSE 0
#define MSOSM_SIM_GAUSSIAN 1
#define MSOSM_SIM_IMPULSES 2
typedef struct msosm_sim_s msosm_sim_t;
int msosm_sim_create(float bw, float f0, float dm, float period, msosm_sim_t **out);
int msosm_sim_set_pulse(msosm_sim_t *s, int kind, float duty);
int msosm_sim_set_noise(msosm_sim_t *s, int enable, float snr_db);
int msosm_sim_set_seed(msosm_sim_t *s, unsigned long long seed);
int msosm_sim_info(const msosm_sim_t *s, unsigned long long *period_samples, unsigned long long *nd,
                   double *signal_power, double *noise_sigma);
int msosm_sim_generate(msosm_sim_t *s, unsigned long long n, int out_format, float scale, void *out, void *stream);
unsigned long long msosm_sim_position(const msosm_sim_t *s);
const char *msosm_sim_last_error(const msosm_sim_t *s);
int msosm_sim_destroy(msosm_sim_t *s);
int msosm_awgn(unsigned long long seed, unsigned long long first, unsigned long long n, float mean, float stddev,
               float *out, void *stream);

/* ---- overlap-save filtering without device allocation --------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate
 * device memory when they filter -- real-time loops that allocate everything at
 * start-up because cudaMalloc/cudaFree synchronise the device and can miss a
 * buffer deadline, and plug-ins inside a host application that owns the GPU's
 * memory budget.  Filters `count` overlapping windows of one DM with response H:
 *   x   device complex64, (count+1)*M samples (M = fftpoint/2); the first M are
 *       the history the first window overlaps
 *   H   device complex64, fftpoint bins (e.g. msosm_plan_response's output)
 *   out device complex64, count*M samples: window b's samples M..2M-1 of
 *       IFFT(FFT(x[b*M .. b*M+2M)) * H) / fftpoint, as msosm_process computes them
 * Intermediates live in a fixed file-scope device array of 18,939,904 bytes that
 * every GPU loading the library holds until exit; no cudaMalloc/cudaFree or other
 * allocating call is made.  Limits: fftpoint a power of two in [2^8, 2^20] and
 * count*fftpoint <= 2^20; larger requests return MSOSM_ERR_UNSUPPORTED with a
 * message on stderr.  The first call on each device looks up the array's device
 * address (one-time set-up), so make it before any stream capture.  The address
 * is kept for the life of the process: do not use this entry point on a device
 * after cudaDeviceReset.  x, H and out must be device memory of the current
 * device (or managed memory).  All calls share the array and it keeps the last
 * call's contents: calls that overlap on the GPU race, so order them on one
 * stream. */
int msosm_osm_filter_noalloc(const void *x, const void *H, int fftpoint, int count, void *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MSOSM_GB300_H */
