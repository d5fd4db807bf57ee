// Internal host/device interfaces of libusgb (not part of the C ABI).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace usgb {

constexpr int kPrepThreads = 512;
constexpr int kMaxFFTStages = 24;
constexpr unsigned kTwiddleSplit = 128;   // two-level twiddle tables: W^m = hi[m / 128] * lo[m % 128]
constexpr unsigned kHilbertSkip = 0xFFFFFFFFu;
// FIR taps copied into the launch parameters for the specialised FIR shapes
// (U x tapsStride: 8 phases x 28 at most), read there as constant-bank
// operands instead of shared-memory loads.
constexpr unsigned kParamTaps = 224;
constexpr unsigned kHilbertSwap = 0x80000000u;
// FP32 delays (a sum of two rounded products of rounded distances) are off by
// at most about 8 * 2^-24 * d samples; above 32768 samples that can exceed
// 1/64 sample, and the staged kernel switches the tile to FP64 geometry.
constexpr float kDeepDelaySamples = 32768.0f;

// One launch of the signal-preparation kernel over `numSignals` A-scans.
struct PrepParams {
	const float* rf;             // numSignals x ns, float32
	void* out;                   // numSignals x outStride samples (storage type)
	size_t outStride;            // samples per A-scan in `out` (>= L)
	unsigned numSignals;
	unsigned ns;                 // samples per A-scan at fs
	unsigned U;                  // upsampling factor (1: none)
	unsigned L;                  // ns * U
	unsigned tapsPerPhase;       // 2K + 1 (1 when U == 1)
	unsigned tapsStride;         // tapsPerPhase rounded up to a multiple of 4
	const float* polyTaps;       // U x tapsStride, polyTaps[r][t] = h[r + tU] (zero padded)
	unsigned deadZone;           // first sample of the DC mean
	float paramTaps[kParamTaps]; // polyTaps again when U * tapsStride <= kParamTaps (single-frame launches)
	float outScale;              // applied before storage (1 for FP32)
	// Hilbert FFT (analytic path): M = N/2 complex points.
	unsigned M;
	int numStages;
	int radix[kMaxFFTStages];    // DIF order
	unsigned long long divMagic[kMaxFFTStages];  // floor(b / sub_s) = (b * divMagic[s]) >> 40
	const float2* tw;            // twLo (128) then twHi (ceil(M/128)): exp(-2 pi i m / M)
	unsigned twHiCount;
	// Hilbert pass over the pairs (k, M - k) in digit-reversed position
	// order: entry p < hilbCount = ((cos, sin)(pi k_lo / M), code, 0) with
	// code = the partner's position q > p (| kHilbertSwap when p holds M - k_lo
	// rather than k_lo), p itself for k = 0 and k = M / 2, or kHilbertSkip
	// when the pair was visited from the partner's lower position.
	const float4* hilb;
	unsigned hilbCount;
	// Per-stage twiddle tables (stage s >= 1: W_Ms^j, j < Ms / radix, at
	// stw + stwOffset[s]); null when they do not fit in shared memory, and
	// every stage then reads the two-level table.
	const float2* stw;
	unsigned stwCount;
	unsigned stwOffset[kMaxFFTStages];
	// DC removal inside the FIR pass (single-frame launches of the
	// specialised FIR shapes): dcCoef[b] is the sum of the FIR taps through
	// which input sample b reaches an output in [deadZone, L), so the mean of
	// [deadZone, L) is sum_b rf[b] dcCoef[b] / (L - deadZone), known before
	// the FIR runs. Null: the mean is taken from the FIR outputs.
	const float* dcCoef;
	// The rows of `rf` are device memory, 16-byte aligned, ns a multiple of 4:
	// they may be fetched with bulk copies.
	unsigned rfBulk;
	// Tensor-memory columns of a single-frame analytic block (the real parts
	// parked there during the FFTs), 0: two store passes instead. Set by the
	// launch.
	unsigned tmemCols;
	unsigned* errWord;           // device status word of the bounded waits, or null
};

size_t prep_smem_bytes(const PrepParams& p, bool analytic);
// Threads per preparation block for `smem` bytes of shared memory a block:
// 128 when four blocks fit on an SM, 256 when two fit, else 512.
int prep_threads(size_t smem);
// Tensor-memory columns of a batch preparation launch of `smem` bytes a block
// whose longest A-scan has maxL samples (the 512-thread form only), else 0.
unsigned prep_batch_tmem_columns(size_t smem, unsigned maxL, bool analytic);
// Envelope (|analytic signal|, no DC removal) of p.numSignals real sequences of
// p.ns = p.L samples (U = 1, one FIR tap of 1), float output, p.outStride apart.
cudaError_t launch_envelope(const PrepParams& p, cudaStream_t stream);
cudaError_t launch_prep(const PrepParams& p, int storage, bool analytic, cudaStream_t stream);
// Whether launch_prep runs the persistent single-frame kernel (DC weights
// given, specialised FIR shape), and the shared memory a block of it needs.
bool prep_uses_stream(const PrepParams& p);
size_t prep_stream_smem_bytes(const PrepParams& p, bool analytic);

// One launch of the delay-and-sum kernel over the grid points of one frame.
struct DasParams {
	const void* sig;             // numTx x numRx x sigStride samples (storage type)
	size_t sigStride;            // samples per A-scan
	unsigned L;                  // valid samples per A-scan
	unsigned numTx, numRx;
	const float* txXY;           // numTx (x, y)
	const float* rxXY;           // numRx (x, y)
	const float* apod;           // numRx
	const float* grid;           // npix (x, y, z)
	unsigned npix, ncols, nrows;
	float invCT;                 // fs * U / c
	float signalOffset;          // fs * U * peakOffset / fc
	float valueCoef;             // 1 / (numTx * numRx)
	float invScale;              // 1 / storage scale
	float pcfFactor;             // gamma / sigma0
	float scfP;
	// Delay precision of the staged kernel: 0 = FP64 geometry for the tiles
	// whose FP32 delay error could exceed 1/64 sample (largest delay above
	// kDeepDelaySamples), FP32 elsewhere; 1 = FP32 everywhere; 2 = FP64
	// everywhere. invCTd / signalOffsetd are invCT / signalOffset in double.
	int delayMode;
	double invCTd;
	double signalOffsetd;
	float* value;
	float* factor;
	unsigned* errWord;
	// Bounded waits of the staged kernels give up after waitLimitNs
	// nanoseconds (0: the default of 2 s). testSkipStage = k > 0 makes the
	// window producer of every pixel tile leave its k-th stage unarmed, so
	// that the consumers' wait for it runs out (the timeout path's test
	// hook; 0 in normal use).
	unsigned long long waitLimitNs;
	unsigned testSkipStage;
	// Staged kernels: columns (32; 64 for the receiver-group kernel's wide
	// tiles) and rows of the pixel tile, bytes per pipeline stage, number of
	// stages (2..16).
	unsigned tileCols;
	unsigned tileRows;
	unsigned stageBytes;
	unsigned stages;
	// Receiver-group kernel: grid points per consumer thread (0 or 1: one;
	// 2: two neighbouring rows, the tile then spans 2 x tileRows rows).
	unsigned pointsPerThread;
};

// variant 0: plain kernel; 1: staged kernel; 2: receiver-group kernel
// (32-column tiles); 3: receiver-group kernel, 64-column tiles; 4: as 3 with
// two grid points (neighbouring rows) per consumer thread.
cudaError_t launch_das(const DasParams& p, int storage, int cf, bool analytic, int variant, cudaStream_t stream);
cudaError_t launch_das_staged(const DasParams& p, int storage, int cf, bool analytic, cudaStream_t stream);
// variant 2: receiver-group kernel (usgb_das_group.cu).
cudaError_t launch_das_group(const DasParams& p, int storage, int cf, bool analytic, cudaStream_t stream);
size_t das_group_smem_bytes(unsigned numTx, unsigned numRx, unsigned tileCols, unsigned tileRows, unsigned capBytes,
		unsigned stages);
// Tile columns of a delay-and-sum variant.
inline unsigned das_tile_cols(int variant) { return variant >= 3 ? 64u : 32u; }
// Grid-point rows of a tile per thread row (variant 4: two).
inline unsigned das_points_per_thread(int variant) { return variant == 4 ? 2u : 1u; }

// ---------------------------------------------------------------------------
// Batched (multi-frame) launches: persistent blocks walk the work items of
// every frame; descriptors live in device memory so a captured graph can be
// replayed with new frames.
// ---------------------------------------------------------------------------
struct BatchHeader {
	unsigned count;          // frames in the batch
	unsigned totalSignals;   // sum of A-scans (prep work items)
	unsigned totalTiles;     // sum of DAS tiles
	unsigned pad;
};

struct BatchPrepFrame {
	PrepParams prep;
	unsigned signalBegin;    // first global A-scan index of the frame
	unsigned pad[3];
};

struct BatchDasFrame {
	DasParams das;
	unsigned tileBegin;      // first global tile index of the frame
	unsigned tilesX;         // tiles per row of tiles
	int cf;
	unsigned pad;
};

struct BatchDasConfig {
	unsigned maxTx, maxRx;   // layout limits of the shared memory
	unsigned tileCols, tileRows, stageBytes, stages;
	unsigned blocks;         // persistent grid size (0: as many blocks as the SMs hold)
	unsigned pointsPerThread;  // receiver-group kernel: 1, or 2 (64 x 2*tileRows tiles)
};

cudaError_t launch_prep_batch(const BatchPrepFrame* frames, const BatchHeader* hdr, size_t smem, unsigned blocks,
		int storage, bool analytic, cudaStream_t stream);
cudaError_t launch_das_staged_batch(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		int storage, bool analytic, cudaStream_t stream);
size_t das_staged_smem_bytes(unsigned numTx, unsigned numRx, unsigned tileRows, unsigned capBytes, unsigned stages);
cudaError_t launch_das_group_batch(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		int storage, bool analytic, cudaStream_t stream);

}  // namespace usgb
