/*
 * libusgb: GB300-native (sm_103a) STA/TFM delay-and-sum imaging, C ABI.
 *
 * Drop-in replacement for the signal-preparation and delay-and-sum stages
 * that sit behind the reference's processor plugin interface
 * ArrayProcessor<TPoint>::prepare/process
 * (src/user/processor/ArrayProcessor.h:28-40), i.e. for
 *   VectorialSTAProcessor<float, XYZValueFactor<float>>   src/user/processor/VectorialSTAProcessor.h:58-341
 *   VectorialSTACUDAProcessor                             src/user/processor/VectorialSTACUDAProcessor.h:63-127
 *   Vectorial3DSTAProcessor<float>                        src/user/processor/Vectorial3DSTAProcessor.h:51-253
 *   DefaultSTAProcessor<float, XYZValueFactor<float>>     src/user/processor/DefaultSTAProcessor.h:50-227
 *
 * Plain C types only. Every function returns a usgb_status; the message of
 * the last failure is available from usgb_last_error(). No exceptions cross
 * this boundary. A context is not thread-safe; use one per thread/stream
 * (the reference's processors are likewise not re-entrant).
 */
#ifndef USGB_H
#define USGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The first three map to the reference's exception types
 * (src/util/Exception.h): InvalidParameterException, InvalidValueException,
 * InvalidStateException; USGB_ERR_CUDA to CUDAException (src/util/CUDAUtil.h:13-16). */
typedef enum usgb_status {
	USGB_OK = 0,
	USGB_ERR_INVALID_PARAMETER = 1,
	USGB_ERR_INVALID_VALUE = 2,
	USGB_ERR_INVALID_STATE = 3,
	USGB_ERR_CUDA = 4,
	USGB_ERR_UNSUPPORTED = 5,
	USGB_ERR_OUT_OF_MEMORY = 6,
	USGB_ERR_DEVICE_TIMEOUT = 7
} usgb_status;

/* Which reference processor's arithmetic to follow. */
typedef enum usgb_signal_path {
	/* VectorialSTAProcessor / Vectorial3DSTAProcessor: Kaiser-sinc upsampling
	 * by `upsampling`, DC removal, Hilbert analytic signal, rx apodization,
	 * value = |sum|. */
	USGB_PATH_ANALYTIC = 0,
	/* DefaultSTAProcessor: fixed 4x FIR, DC removal, real samples, no
	 * apodization, value = signed sum (`upsampling` must be 4). */
	USGB_PATH_REAL = 1
} usgb_signal_path;

/* Coherence factor written to `factor` (1 when none). */
typedef enum usgb_coherence {
	USGB_CF_NONE = 0,
	USGB_CF_PCF = 1, /* phase coherence factor, src/util/CoherenceFactor.h:240-296 */
	USGB_CF_SCF = 2, /* sign coherence factor, src/util/CoherenceFactor.h:198-236 (on Re for the analytic path) */
	USGB_CF_MF = 3   /* |sum s|^2 / (N sum |s|^2); no counterpart in the reference */
} usgb_coherence;

/* Storage type of the prepared signal tensor (accumulation is always FP32). */
typedef enum usgb_storage {
	USGB_STORE_F32 = 0,
	USGB_STORE_F16 = 1,
	USGB_STORE_BF16 = 2
} usgb_storage;

/* Precision of the per-pixel delays in the staged delay-and-sum kernel. The
 * reference computes them in FP32 (VectorialSTAProcessor.h:265-277); FP32
 * delays of d samples are off by up to about 8 * 2^-24 * d samples, which
 * exceeds 1/64 sample beyond d = 32768 (deep grids at high upsampling). */
typedef enum usgb_delay_precision {
	USGB_DELAY_AUTO = 0, /* FP64 geometry for the pixel tiles whose largest delay exceeds 32768 samples, FP32 elsewhere */
	USGB_DELAY_FP32 = 1, /* FP32 everywhere, as the reference */
	USGB_DELAY_FP64 = 2  /* FP64 geometry everywhere */
} usgb_delay_precision;

/*
 * Frame description. Mirrors the constructor arguments of
 * VectorialSTAProcessor(config, acquisition, upsamplingFactor, coherenceFactor,
 * peakOffset, rxApod) (src/user/processor/VectorialSTAProcessor.h:61-67) with
 * STAConfiguration's fields (src/user/configuration/STAConfiguration.h:29-48);
 * element positions are given explicitly so that the linear array
 * (ArrayGeometry::getElementXCentered2D, src/util/ArrayGeometry.h:37-49) and
 * the 2D matrix array (ArrayUtil::calculateElementPositions,
 * src/util/ArrayUtil.h:51-70) use the same entry points.
 */
typedef struct usgb_sta_params {
	uint32_t num_tx;            /* active transmit elements (lastTxElem - firstTxElem + 1) */
	uint32_t num_rx;            /* receive elements */
	uint32_t num_samples;       /* samples per A-scan at sampling_frequency */
	uint32_t upsampling;        /* upsamplingFactor, 1..64 (4 for USGB_PATH_REAL) */
	uint32_t signal_path;       /* usgb_signal_path */
	float sampling_frequency;   /* Hz */
	float propagation_speed;    /* m/s */
	float center_frequency;     /* Hz */
	float peak_offset;          /* peakOffset, in periods of center_frequency */
	float dead_zone_m;          /* m */
	const float* tx_xy;         /* host, num_tx (x, y) pairs, m */
	const float* rx_xy;         /* host, num_rx (x, y) pairs, m */
	const float* rx_apod;       /* host, num_rx weights; NULL = all ones */
	uint32_t coherence;         /* usgb_coherence */
	float pcf_gamma;            /* phase_coherence_factor_gamma */
	float scf_p;                /* sign_coherence_factor_p */
	uint32_t storage;           /* usgb_storage */
	float storage_scale;        /* samples are multiplied by this before FP16/BF16 storage; 0 = 1 */
} usgb_sta_params;

typedef struct usgb_ctx usgb_ctx;

/* Creates a context on the current CUDA device (checks the parameters, builds
 * the FIR and FFT tables, allocates the per-frame device buffers). */
int usgb_create(const usgb_sta_params* params, usgb_ctx** ctx);
void usgb_destroy(usgb_ctx* ctx);
/* Message of the last failure on `ctx` (or of the last failed usgb_create on
 * this thread when ctx is NULL). Never NULL. */
const char* usgb_last_error(const usgb_ctx* ctx);

/* Image grid: ncols * nrows points (x, y, z), column-major like the reference's
 * Matrix<XYZValueFactor> (point(col, row) at index col * nrows + row,
 * src/util/Matrix.h:188-198). Host pointer. */
int usgb_set_grid(usgb_ctx* ctx, const float* xyz, uint32_t ncols, uint32_t nrows);

/* RF of one transmit event, as STAAcquisition::execute delivers it
 * (src/user/acquisition/STAAcquisition.h:36): num_rx rows of num_samples.
 * tx is the index among the active transmit elements. Host pointer; the data
 * is copied into the context's pinned staging buffer. */
int usgb_submit_rf(usgb_ctx* ctx, uint32_t tx, const float* rf, uint32_t num_rx, uint32_t num_samples);

/* Forms the image from the submitted RF, like ArrayProcessor::process:
 * value = |sum| / (num_tx * num_rx) (signed sum for USGB_PATH_REAL) and
 * factor = coherence factor (1 when none), both ncols * nrows floats in the
 * grid's order, host pointers. Synchronous. */
int usgb_process(usgb_ctx* ctx, float* value, float* factor);

/* Device-resident forms (asynchronous on the context's stream). d_rf holds
 * num_tx * num_rx * num_samples floats; d_value and d_factor ncols * nrows. */
int usgb_set_stream(usgb_ctx* ctx, void* cuda_stream);
int usgb_set_grid_device(usgb_ctx* ctx, const float* d_xyz, uint32_t ncols, uint32_t nrows);
int usgb_process_device(usgb_ctx* ctx, const float* d_rf, float* d_value, float* d_factor);

/* One whole frame from host memory: rf = num_tx * num_rx * num_samples floats
 * (transmit-major, as the submitted rows), value / factor = ncols * nrows
 * floats (factor may be NULL). Synchronous, like usgb_process. On devices
 * that reach pageable host memory through the host's page tables (Grace-based
 * GB300 systems) the kernels read the RF and write the images in place, with
 * no staging copy; elsewhere the RF is copied in and the images out. No
 * counterpart in the reference (its acquisition delivers one transmit event
 * at a time, usgb_submit_rf). */
int usgb_process_rf(usgb_ctx* ctx, const float* rf, float* value, float* factor);

/* Direct host-memory access of usgb_process_rf: enable = 0 forces the copy
 * path; enable = 1 fails with USGB_ERR_UNSUPPORTED where the device cannot.
 * usgb_get_host_direct reports whether it is available and enabled. */
int usgb_set_host_direct(usgb_ctx* ctx, int enable);
int usgb_get_host_direct(const usgb_ctx* ctx, int* available, int* enabled);

/* The two stages separately. d_signals holds num_tx * num_rx A-scans of
 * signal_stride samples (complex (re, im) pairs on the analytic path, reals on
 * the real path) in the context's storage type. */
int usgb_prepare_signals_device(usgb_ctx* ctx, const float* d_rf, void* d_signals);
int usgb_delay_and_sum_device(usgb_ctx* ctx, const void* d_signals, float* d_value, float* d_factor);

/* Sizes: signal_length = num_samples * upsampling; fft_size = Hilbert FFT
 * length N (0 on the real path); signal_stride = samples per A-scan in the
 * signal tensor; signal_bytes = bytes of the whole tensor. */
int usgb_signal_info(const usgb_ctx* ctx, uint32_t* signal_length, uint32_t* fft_size,
		uint32_t* signal_stride, size_t* signal_bytes);

/* Selects the delay-and-sum kernel: 0 = plain (one thread per point, gathers
 * from global memory), 1 = staged (per tile of 32 columns x tile_rows rows,
 * the A-scan windows the tile needs are bulk-copied into a shared-memory ring
 * of `stages` stages of stage_bytes each; receiver by receiver, transmit
 * delays in a per-point table), 2 = receiver-group (the same ring, filled
 * receiver group by receiver group; a group's receive delays and sums stay in
 * registers, no per-point table, so arrays of hundreds of elements stage as
 * well), 3 = receiver-group on tiles of 64 columns x tile_rows (1 to 8) rows
 * (windows only a little longer for twice the points: fewer bytes and half
 * the copies staged per frame), 4 = as 3 with two grid points (neighbouring
 * rows) per consumer thread, tiles of 64 columns x 2 * tile_rows rows (twice
 * the independent loads per warp between two stage waits, fewer bytes staged
 * per point). 0 for tile_rows / stage_bytes / stages keeps
 * the current value. New
 * contexts start with the receiver-group kernel (32 x 4 tiles, 2 x 32 KiB)
 * where it fits; setting a grid of at least 1.5 tiles of 64 x 16 points per
 * SM then selects variant 4 with 2 x 100 KiB stages and tile_rows in [5, 8]
 * for the fewest whole waves of tiles (512 x 512 on 152 SMs: 7, 64 x 14
 * tiles), else one of at least two 64-column tiles per SM variant 3 (64 x 8
 * with 2 x 100 or 96 KiB stages, else 64 x 4 with 2 x 48 KiB) where it fits,
 * unless a variant was set here or by usgb_autotune_das. */
int usgb_set_das_variant(usgb_ctx* ctx, int variant, uint32_t tile_rows, uint32_t stage_bytes, uint32_t stages);
int usgb_get_das_config(const usgb_ctx* ctx, int* variant, uint32_t* tile_rows, uint32_t* stage_bytes,
		uint32_t* stages);

/* Delay precision of the staged kernel (usgb_delay_precision; new contexts:
 * USGB_DELAY_AUTO). FP64 tiles compute each pixel's transmit and receive
 * delays in double and sum them as 32-bit fixed point with 2^-10 sample
 * resolution. No counterpart in the reference, which is FP32 throughout; the
 * plain kernel (variant 0) always uses FP32. */
int usgb_set_delay_precision(usgb_ctx* ctx, uint32_t mode);

/* Times every staged configuration that fits (tile rows x stage bytes x
 * stages, plus the plain kernel) on the given prepared signals, `iterations`
 * runs each, keeps the fastest on the context and returns its time. */
int usgb_autotune_das(usgb_ctx* ctx, const void* d_signals, float* d_value, float* d_factor, uint32_t iterations,
		float* best_ms);

/* Waits for the context's stream and reports a device-side error (a bounded
 * wait that gave up) as USGB_ERR_DEVICE_TIMEOUT. */
int usgb_synchronize(usgb_ctx* ctx);

/* Test hook of the timeout path (no counterpart in the reference). Every
 * wait of the staged delay-and-sum kernels (variants 1-3) is bounded: after
 * its limit the waiting warp records DEVERR_WAIT_TIMEOUT in the context's
 * error word, the kernel winds down once its copies in flight have landed,
 * and usgb_process / usgb_process_rf / usgb_synchronize return
 * USGB_ERR_DEVICE_TIMEOUT; the context stays usable. wait_limit_us sets the
 * limit (0: the default 2 s); skip_stage = k > 0 makes the window producer of
 * every pixel tile leave its k-th stage unarmed, so the consumers' wait for it
 * runs out. skip_stage = 0 and wait_limit_us = 0 restore normal operation. */
int usgb_set_wait_test(usgb_ctx* ctx, uint32_t wait_limit_us, uint32_t skip_stage);

/*
 * Image post-processing (the reference's dB image: envelope along each image
 * column, ParallelHilbertEnvelope<float>::calculateDim2Value,
 * src/parallel/ParallelHilbertEnvelope.h:83-95, then Util::linearToDecibels,
 * src/util/Util.h:600-613). A usgb_post holds the FFT tables for columns of
 * num_samples values (the grid's nrows).
 *   usgb_post_envelope_device: d_out[c][n] = |analytic signal of column c|[n]
 *     for num_columns columns of num_samples floats (column-major images as
 *     the processors write them); d_in and d_out may be the same buffer.
 *   usgb_post_decibels_device: in place, v / max|v| (unless the maximum is 0),
 *     then 20 log10(v), or min_db at or below 10^(min_db / 20).
 */
typedef struct usgb_post usgb_post;
int usgb_post_create(uint32_t num_samples, usgb_post** post);
void usgb_post_destroy(usgb_post* post);
const char* usgb_post_last_error(const usgb_post* post);
int usgb_post_envelope_device(usgb_post* post, const float* d_in, float* d_out, uint32_t num_columns, void* stream);
int usgb_post_decibels_device(usgb_post* post, float* d_data, size_t n, float min_db, void* stream);

/*
 * One frame without any device allocation. No counterpart in the reference:
 * it exists for callers that must not allocate device memory while they run,
 * e.g. a host that has already given nearly all GPU memory to its own pool
 * (an allocation by this library would fail or fragment it) or an
 * acquisition loop with a fixed latency budget. The caller passes the RF
 * (num_tx * num_rx * num_samples floats), the grid (ncols * nrows (x, y, z))
 * and the outputs (ncols * nrows floats each), all device pointers; the
 * tables, element positions and prepared signal tensor live in a fixed 64 MiB
 * device array inside the library, which every GPU that loads the library
 * keeps until the process exits. Frames that need more (tables plus
 * num_tx * num_rx * signal length samples) are rejected with
 * USGB_ERR_INVALID_VALUE and a message saying so. Every call shares the array
 * and finds there what the previous call left; each call rewrites what it
 * uses, but calls whose GPU work overlaps race on it, so order them. The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture.
 * Parameters are checked by the same rules, with the same messages, as
 * usgb_create; grids above 2^31 points are rejected ("Grid too large.").
 * d_status: optional device word for device-side failures. When given, the
 * call clears it, the kernels set it (bit 0: a bounded delay-and-sum wait gave
 * up, the image is incomplete) and the call returns without waiting for the
 * GPU (asynchronous on cuda_stream, NULL = default stream); read the word with
 * the images. When NULL, the call waits for its work on cuda_stream and
 * returns USGB_ERR_DEVICE_TIMEOUT itself on such a failure. On failure the
 * message is copied into error_message (error_capacity bytes, may be NULL).
 */
int usgb_process_frame_noalloc(const usgb_sta_params* params, const float* d_rf, const float* d_grid_xyz,
		uint32_t ncols, uint32_t nrows, float* d_value, float* d_factor, uint32_t* d_status, void* cuda_stream,
		char* error_message, size_t error_capacity);

/*
 * Batches: many frames (different element counts, sample counts, grids and
 * coherence factors; one storage type and signal path) in two persistent
 * launches, one over every A-scan of every frame (preparation) and one over
 * every grid tile of every frame (staged delay-and-sum). Each frame is a
 * context (geometry, tables, grid, signal tensor) plus its device RF and
 * outputs. Frame descriptors are copied to the device at each run, so with
 * use_graph the two launches are captured once into a CUDA graph and the
 * graph is replayed for every later batch (re-captured only when a batch
 * needs more shared memory than the captured one). A batch object may have
 * one run in flight; usgb_batch_run waits for the previous run's descriptor
 * copy before refilling its descriptors.
 */
typedef struct usgb_batch usgb_batch;
typedef struct usgb_batch_item {
	usgb_ctx* ctx;          /* frame: parameters, tables, grid, signal tensor */
	const float* d_rf;      /* device RF, num_tx * num_rx * num_samples */
	float* d_value;         /* device outputs, ncols * nrows each */
	float* d_factor;
} usgb_batch_item;
int usgb_batch_create(uint32_t max_frames, uint32_t max_elements, uint32_t max_signal_length, usgb_batch** batch);
void usgb_batch_destroy(usgb_batch* batch);
const char* usgb_batch_last_error(const usgb_batch* batch);
int usgb_batch_set_das_config(usgb_batch* batch, uint32_t tile_rows, uint32_t stage_bytes, uint32_t stages);
/* Delay-and-sum kernel of the batch: 2 = receiver-group (default), 3 =
 * receiver-group on 64-column tiles, 4 = receiver-group on 64 x 2*tile_rows
 * tiles with two points per thread (tile_rows 4, 7 or 8), 1 = staged. */
int usgb_batch_set_das_variant(usgb_batch* batch, int variant);
int usgb_batch_run(usgb_batch* batch, const usgb_batch_item* items, uint32_t count, void* cuda_stream, int use_graph);
int usgb_batch_synchronize(usgb_batch* batch);

/*
 * Single-term 3D processors: one prepared A-scan per term, so each grid point
 * sums one linearly interpolated sample per signal (per signal and
 * acquisition for the synthetic-y array) instead of one per tx x rx pair.
 * Drop-in for
 *   Vectorial3DT1R1SAFTProcessor<float>    src/user/processor/Vectorial3DT1R1SAFTProcessor.h:51-236
 *     (prepare/process :120-236; delays :200-220)
 *   Vectorial3DTnRnProcessor<float>        src/user/processor/Vectorial3DTnRnProcessor.h:51-282
 *     (setTxDelays :137-146, prepare :148-161, process :163-282)
 *   SynthYVectorial3DTnRnProcessor<float>  src/user/processor/SynthYVectorial3DTnRnProcessor.h:51-305
 *     (getAcqData :169-205, process(firstAcq, lastAcq, grid) :207-305)
 * The signals go through the same preparation as the STA processors
 * (upsampling, DC removal, analytic signal); value = |sum of terms| /
 * num_signals (times 1 / number of acquisitions of the window for the
 * synthetic-y array) and factor = the coherence factor over all terms.
 */
typedef enum usgb_single_mode {
	USGB_SINGLE_T1R1_SAFT = 0,    /* per-signal tx and rx element: delay = offset + |tx - p| / c + |rx - p| / c */
	USGB_SINGLE_TNRN = 1,         /* one focused or diverging transmit (virtual source), rx apodization */
	USGB_SINGLE_SYNTH_Y_TNRN = 2  /* TnRn acquisitions at several y positions, summed as one array in y */
} usgb_single_mode;

/* Mirrors the constructor arguments (config, acquisition, upsamplingFactor,
 * coherenceFactor, peakOffset[, rxApod]) with SA3DConfiguration /
 * TnRnConfiguration's fields (src/user/configuration/SA3DConfiguration.h:37-57,
 * TnRnConfiguration.h:34-53). */
typedef struct usgb_single_params {
	uint32_t mode;              /* usgb_single_mode */
	uint32_t num_signals;       /* T1R1: active elements (activeTxElem.size() == activeRxElem.size()); TnRn: numElements */
	uint32_t num_samples;       /* samples per A-scan at sampling_frequency */
	uint32_t upsampling;        /* 1..64 */
	float sampling_frequency;   /* Hz */
	float propagation_speed;    /* m/s */
	float center_frequency;     /* Hz */
	float peak_offset;          /* periods of center_frequency */
	float dead_zone_m;          /* m */
	/* host (x, y) pairs, m. T1R1: num_signals pairs, txElemPos[base + activeTxElem[i]].
	 * TnRn: at least one pair; pair 0 = txElemPos[baseElement], the first element of the group. */
	const float* tx_xy;
	/* host, num_signals (x, y) pairs: T1R1 rxElemPos[base + activeRxElem[i]]; TnRn rxElemPos[baseElement + i]. */
	const float* rx_xy;
	/* host, num_signals weights. TnRn: required (the reference rejects a list of
	 * the wrong size); T1R1: must be NULL (no apodization). */
	const float* rx_apod;
	uint32_t coherence;         /* usgb_coherence (USGB_CF_NONE / PCF / SCF on Re / MF) */
	float pcf_gamma;
	float scf_p;
	uint32_t storage;           /* usgb_storage of the prepared signals */
	float storage_scale;        /* samples are multiplied by this before FP16/BF16 storage; 0 = 1 */
	uint32_t max_acquisitions;  /* synthetic y: acquisitions kept on the device (a ring); others: 0 or 1 */
} usgb_single_params;

typedef struct usgb_single usgb_single;
int usgb_single_create(const usgb_single_params* params, usgb_single** single);
void usgb_single_destroy(usgb_single* single);
const char* usgb_single_last_error(const usgb_single* single);  /* NULL: last failed create on this thread */
int usgb_single_set_stream(usgb_single* single, void* cuda_stream);

/* setTxDelays(focusX, focusY, focusZ, txDelays): the focus (focus_z <= 0: a
 * virtual source behind the array) and the group's transmit delays in s
 * (ArrayUtil::calculateTx3DFocusDelay, src/util/ArrayUtil.h:100-144); only
 * tx_delays[0] enters the image. TnRn modes; processing without it is
 * USGB_ERR_INVALID_STATE ("Empty tx delay list."), as the reference's prepare. */
int usgb_single_set_tx_delays(usgb_single* single, float focus_x, float focus_y, float focus_z,
		const float* tx_delays, uint32_t count);

/* Grid, column-major as in usgb_set_grid (host or device pointer). */
int usgb_single_set_grid(usgb_single* single, const float* xyz, uint32_t ncols, uint32_t nrows);
int usgb_single_set_grid_device(usgb_single* single, const float* d_xyz, uint32_t ncols, uint32_t nrows);

/* T1R1 / TnRn: forms the image of one acquisition, rf = num_signals rows of
 * num_samples (host; synchronous) or d_rf (device; asynchronous on the stream). */
int usgb_single_process(usgb_single* single, const float* rf, float* value, float* factor);
int usgb_single_process_device(usgb_single* single, const float* d_rf, float* d_value, float* d_factor);

/* Synthetic y. usgb_single_add_acquisition(_device) prepares one acquisition
 * (num_signals rows of num_samples) taken at `y` and appends it as number
 * count++ (getAcqData(y)); the device keeps the last max_acquisitions.
 * usgb_single_process_window(_device) forms the image of acquisitions
 * first_acq..last_acq (process(firstAcq, lastAcq, gridData)): the grid's y is
 * taken relative to the y of acquisition (first_acq + last_acq) / 2, which the
 * reference then writes into every grid point's y. */
int usgb_single_add_acquisition(usgb_single* single, const float* rf, float y);
int usgb_single_add_acquisition_device(usgb_single* single, const float* d_rf, float y);
int usgb_single_num_acquisitions(const usgb_single* single, uint32_t* count);
int usgb_single_process_window(usgb_single* single, uint32_t first_acq, uint32_t last_acq, float* value, float* factor);
int usgb_single_process_window_device(usgb_single* single, uint32_t first_acq, uint32_t last_acq, float* d_value,
		float* d_factor);
int usgb_single_synchronize(usgb_single* single);

/*
 * Two-medium imaging: a linear array in medium 1 (speed c1) images medium 2
 * (speed c2) through an interface given as a list of (x, z) points. Delays
 * follow Fermat's principle (the fastest path through an interface point);
 * each step of a sub-aperture moved across the array adds its delay-and-sum
 * (one transmit element, or STA over several) to a complex image. Drop-in for
 *   VectorialCombinedTwoMediumImagingProcessor<float>
 *     src/user/processor/VectorialCombinedTwoMediumImagingProcessor.h:59-401
 *     (constructor :192-228, process(stepConfigList, interfacePointList,
 *     rxApod, gridXZ, gridValue) :230-401)
 * and the work of VectorialCombinedTwoMediumImagingCUDAProcessor{,2}
 * (src/user/processor/VectorialCombinedTwoMediumImagingCUDAProcessor.h), with
 * the delay search, the signal preparation and every gather on the GPU.
 */
typedef struct usgb_two_medium_params {
	uint32_t num_elements;          /* numElements: elements of one step (receive; and transmit in STA steps) */
	uint32_t num_elements_mux;      /* numElementsMux: elements of the array, pitch apart, centred on x = 0 */
	float pitch;                    /* m */
	float center_frequency;         /* Hz */
	float propagation_speed_1;      /* medium of the array, m/s */
	float propagation_speed_2;      /* imaged medium, m/s */
	float sampling_frequency;       /* Hz */
	uint32_t num_samples;           /* samples per A-scan of the acquisitions (after the start offset cut) */
	uint32_t upsampling;            /* 1..64 */
	float max_fermat_block_size;    /* maxFermatBlockSize, wavelengths; used as an unsigned count, as the reference */
	float peak_offset;              /* periods of center_frequency */
	uint32_t signal_start_offset;   /* samples cut from the start of every A-scan before the acquisitions */
	uint32_t num_acquisitions;      /* acqDataList.size() */
	uint32_t num_tx;                /* transmit events per acquisition (acqDataList[i].n1()) */
	uint32_t coherence;             /* usgb_coherence over the receive terms of a step (the reference: none or PCF) */
	float pcf_gamma;
	float scf_p;
	uint32_t storage;               /* usgb_storage of the prepared signals */
	float storage_scale;            /* samples are multiplied by this before FP16/BF16 storage; 0 = 1 */
} usgb_two_medium_params;

/* StepConfiguration: acquisition index, first element of the sub-aperture,
 * transmit elements first..last relative to it (all steps one element, or
 * all several). */
typedef struct usgb_two_medium_step {
	uint32_t base_elem_idx;
	uint32_t base_elem;
	uint32_t first_tx_elem;
	uint32_t last_tx_elem;
} usgb_two_medium_step;

typedef struct usgb_two_medium usgb_two_medium;
int usgb_two_medium_create(const usgb_two_medium_params* params, usgb_two_medium** tm);
void usgb_two_medium_destroy(usgb_two_medium* tm);
const char* usgb_two_medium_last_error(const usgb_two_medium* tm);  /* NULL: last failed create on this thread */
int usgb_two_medium_set_stream(usgb_two_medium* tm, void* cuda_stream);

/* process(): rf = the acquisitions (num_acquisitions x num_tx x num_elements x
 * num_samples floats), interface_xz = num_interface (x, z) pairs, rx_apod =
 * num_elements weights, grid_xz = ncols x nrows (x, z) pairs (column-major,
 * rows evenly spaced in z), value = ncols x nrows complex (re, im) pairs;
 * points above the interface are 0. Host pointers, synchronous; the _device
 * form takes device pointers (steps stay on the host) and runs asynchronously
 * on the stream. */
int usgb_two_medium_process(usgb_two_medium* tm, const float* rf, const usgb_two_medium_step* steps, uint32_t num_steps,
		const float* interface_xz, uint32_t num_interface, const float* rx_apod, const float* grid_xz, uint32_t ncols,
		uint32_t nrows, float* value);
int usgb_two_medium_process_device(usgb_two_medium* tm, const float* d_rf, const usgb_two_medium_step* steps,
		uint32_t num_steps, const float* d_interface_xz, uint32_t num_interface, const float* d_rx_apod,
		const float* d_grid_xz, uint32_t ncols, uint32_t nrows, float* d_value);
int usgb_two_medium_synchronize(usgb_two_medium* tm);

/*
 * Saved acquisitions and images: the HDF5 files the reference reads and
 * writes through HDF5Util::load / HDF5Util::save (src/util/HDF5Util.h:181-287):
 * SavedSTAAcquisition's "signal" datasets (FileUtil::txElemSignalsPath,
 * src/util/FileUtil.cpp:58-65: <dir>/signals-base%04u-tx%04u.h5, num_rx rows of
 * num_samples) and Project::saveImageToHDF5 / saveFactorToHDF5 images
 * (image_value.h5 "value", image_factor.h5 "factor", src/Project.h:106-113).
 * Reads HDF5 files of superblock versions 0 and 1 (what libhdf5 writes by
 * default) with one rank-1 or rank-2 32/64-bit floating-point dataset per
 * name, contiguous, compact or chunked, with the shuffle, deflate, LZF and
 * Fletcher-32 filters; writes one contiguous IEEE 64-bit little-endian
 * rank-2 dataset per file. Values are row-major (n1 rows of n2); a rank-1
 * dataset reads as n1 = 1. Host only; no GPU needed. Errors: the message is
 * in usgb_h5_last_error() (this thread).
 */
const char* usgb_h5_last_error(void);
int usgb_h5_dataset_info(const char* path, const char* dataset, uint32_t* rank, uint64_t* n1, uint64_t* n2);
int usgb_h5_read_f64(const char* path, const char* dataset, double* out, size_t capacity, uint64_t* n1, uint64_t* n2);
int usgb_h5_write_f64(const char* path, const char* dataset, const double* data, uint64_t n1, uint64_t n2);

/* Library version string. */
const char* usgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* USGB_H */
