// Two-medium imaging: a linear array in medium 1 images medium 2 through an
// interface sampled as (x, z) points; delays by Fermat's principle, then a
// delay-and-sum per step of a sub-aperture, summed into a complex image.
//   VectorialCombinedTwoMediumImagingProcessor<float>::process
//     src/user/processor/VectorialCombinedTwoMediumImagingProcessor.h:230-401
//   minimum rows                  :256-280 (FermatPrinciple::findNearestPointInXInTwoSteps)
//   medium-1 delays               :282-296
//   CalculateDelays               :403-484 (FermatPrinciple::findMinTimeInTwoSteps, then a walk)
//   PrepareData(WithOneTxElem)    :486-570
//   ProcessColumn(WithOneTxElem)  :572-790
// Four launches besides the preparation: the first imaged row of every
// column, the medium-1 path table (element x interface point), the delay
// table (one thread per column and element walks down the column, each row's
// search starting at the previous row's interface point; columns fastest) and
// the image (one thread per grid point and step, gathering over the step's
// transmit x receive pairs from the table; a warp spans 32 neighbouring
// columns of one row, whose delays differ by a few samples, so both the table
// reads and the sample gathers of a warp fall on few sectors; the warps of a
// block take different steps of the same 32 points). Every delay is rounded as the reference's float arithmetic
// (no contraction, IEEE division and square root), so the searches pick the
// same interface points and each gather reads the same samples with the same
// weight; terms are summed in the reference's order.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/usgb.h"
#include "usgb_common.cuh"
#include "usgb_das_cf.cuh"
#include "usgb_internal.h"
#include "usgb_tables.h"

namespace {

using usgb::CFState;
using usgb::Complex;

constexpr int kTmThreads = 128;

struct TmParams {
	const float2* ifXZ;          // interface points (x, z)
	unsigned nIf;
	const float2* grid;          // ncols x nrows (x, z), point (col, row) at col * nrows + row
	unsigned ncols, nrows;
	unsigned mux;                // elements of the array
	float pitch;
	float lambda2;               // c2 / fc
	unsigned maxBlockWl;         // maximum Fermat block, whole wavelengths
	float invC1, invC2;          // 1 / c1, 1 / c2
	float c2ByC1;                // c2 / c1
	float fsUp;                  // fs * U
	float fsInvC2;               // fs * U / c2
	unsigned* minRow;            // ncols: first imaged row
	float* medium1;              // mux x nIf: element -> interface point, in medium-2 length
	float* delay;                // (row, element, col), samples
	// Image.
	const void* sig;             // (acquisition, tx, rx, sigStride) samples (storage type)
	size_t acqStride, txStride, sigStride;
	unsigned L;
	unsigned numElements;
	const uint4* steps;          // (baseElemIdx, baseElem, firstTxElem, lastTxElem)
	unsigned numSteps;
	const float* apod;           // numElements
	float signalOffset;          // fs * U * (peakOffset / fc) - signalStartOffset * U
	float invScale;
	float pcfFactor, scfP;
	float2* out;                 // ncols x nrows complex
};

// floor(d) and d - floor(d) for 0 <= d < 2^23 (one add rounding toward -inf
// against 2^23); every other d, negatives, infinities and NaN included, gives
// an index outside [0, 2^23) that the unsigned range test rejects.
__device__ __forceinline__ int split_delay(float d, float& frac)
{
	const float t = __fadd_rd(d, 8388608.0f);
	frac = d - (t - 8388608.0f);
	return static_cast<int>(__float_as_uint(t) - 0x4B000000u);
}

__device__ __forceinline__ float hypot_rn(float dx, float dz)
{
	return __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dz, dz)));
}

// ArrayGeometry::getElementX2D with offset 0 (src/util/ArrayGeometry.h:51-63).
__device__ __forceinline__ float element_x(const TmParams& p, unsigned e)
{
	const float xCenter = __fsub_rn(__fdiv_rn(__fmul_rn(static_cast<float>(p.mux - 1U), p.pitch), 2.0f), 0.0f);
	return __fsub_rn(__fmul_rn(static_cast<float>(e), p.pitch), xCenter);
}

// FermatPrinciple::calcBlockSizeForTwoStepSearch (src/util/FermatPrinciple.h:106-115),
// with the interface step taken between the first two points (:250-253 of the processor).
__device__ unsigned fermat_block_size(const TmParams& p)
{
	const float2 a = p.ifXZ[0], b = p.ifXZ[1];
	const float r = hypot_rn(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y));
	const float ideal = static_cast<float>(__dadd_rn(__dsqrt_rn(__ddiv_rn(static_cast<double>(p.nIf), 2.0)), 0.5));
	const float maxBs = __fdiv_rn(__fmul_rn(p.lambda2, static_cast<float>(p.maxBlockWl)), r);
	const float bs = (maxBs < ideal) ? maxBs : ideal;
	const unsigned u = static_cast<unsigned>(bs);
	return u > 2U ? u : 2U;
}

// First imaged row of every column: the interface point nearest in x
// (two steps), then the first row below it (1 when it lies above the grid,
// nrows when below).
__global__ void __launch_bounds__(kTmThreads) tm_min_row_kernel(const __grid_constant__ TmParams p)
{
	const unsigned col = blockIdx.x * blockDim.x + threadIdx.x;
	if (col >= p.ncols) return;
	const unsigned bs = fermat_block_size(p);
	const float2 g0 = p.grid[static_cast<size_t>(col) * p.nrows];
	const float x = g0.x;
	float dxMin = FLT_MAX;
	unsigned idxMin = 0;
	for (unsigned i = 0; i < p.nIf; i += bs) {
		const float dx = fabsf(__fsub_rn(p.ifXZ[i].x, x));
		if (dx < dxMin) {
			dxMin = dx;
			idxMin = i;
		}
	}
	const unsigned iBegin = (idxMin > bs - 1U) ? idxMin - (bs - 1U) : 0U;
	const unsigned iEnd = min(idxMin + bs, p.nIf);
	for (unsigned i = iBegin; i < iEnd; ++i) {
		const float dx = fabsf(__fsub_rn(p.ifXZ[i].x, x));
		if (dx < dxMin) {
			dxMin = dx;
			idxMin = i;
		}
	}
	const float zIdxMin = p.ifXZ[idxMin].y;
	const float zLast = p.grid[static_cast<size_t>(col) * p.nrows + p.nrows - 1U].y;
	unsigned m;
	if (zIdxMin <= g0.y) {
		m = 1U;
	} else if (zIdxMin >= zLast) {
		m = p.nrows;
	} else {
		const float zStep = __fsub_rn(p.grid[1].y, p.grid[0].y);
		m = static_cast<unsigned>(ceilf(__fdiv_rn(__fsub_rn(zIdxMin, g0.y), zStep))) + 1U;
	}
	p.minRow[col] = m;
}

// Medium-1 path element -> interface point, scaled to medium-2 length
// (Geometry::distance2DY0 * c2 / c1).
__global__ void __launch_bounds__(kTmThreads) tm_medium1_kernel(const __grid_constant__ TmParams p)
{
	const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= p.mux * p.nIf) return;
	const unsigned e = t / p.nIf, i = t % p.nIf;
	const float2 q = p.ifXZ[i];
	p.medium1[t] = __fmul_rn(hypot_rn(__fsub_rn(q.x, element_x(p, e)), q.y), p.c2ByC1);
}

// Delays of one column and element down the rows: a two-step Fermat search
// for the first imaged row, then from each row's interface point a walk to
// the neighbour points while the travel time falls.
__global__ void __launch_bounds__(kTmThreads) tm_delay_kernel(const __grid_constant__ TmParams p)
{
	const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= p.ncols * p.mux) return;
	const unsigned col = t % p.ncols, elem = t / p.ncols;  // neighbouring threads: neighbouring columns
	const unsigned r0 = p.minRow[col];
	if (r0 >= p.nrows) return;
	const float2* g = p.grid + static_cast<size_t>(col) * p.nrows;
	const size_t rs = static_cast<size_t>(p.mux) * p.ncols;   // table row stride
	float* out = p.delay + static_cast<size_t>(elem) * p.ncols + col;
	const float x1 = element_x(p, elem);
	unsigned last;
	{
		// FermatPrinciple::findMinTimeInTwoSteps (src/util/FermatPrinciple.h:117-165), z1 = 0.
		const unsigned bs = fermat_block_size(p);
		const float x2 = g[r0].x, z2 = g[r0].y;
		auto time = [&](unsigned i) {
			const float2 q = p.ifXZ[i];
			const float d1 = hypot_rn(__fsub_rn(q.x, x1), __fsub_rn(q.y, 0.0f));
			const float d2 = hypot_rn(__fsub_rn(x2, q.x), __fsub_rn(z2, q.y));
			return __fadd_rn(__fmul_rn(d1, p.invC1), __fmul_rn(d2, p.invC2));
		};
		float tMin = FLT_MAX;
		unsigned idxMin = 0xFFFFFFFFu;
		for (unsigned i = 0; i < p.nIf; i += bs) {
			const float tt = time(i);
			if (tt < tMin) {
				tMin = tt;
				idxMin = i;
			}
		}
		const unsigned iBegin = (idxMin > bs - 1U) ? idxMin - (bs - 1U) : 0U;
		const unsigned iEnd = min(idxMin + bs, p.nIf);
		for (unsigned i = iBegin; i < iEnd; ++i) {
			const float tt = time(i);
			if (tt < tMin) {
				tMin = tt;
				idxMin = i;
			}
		}
		out[r0 * rs] = __fmul_rn(tMin, p.fsUp);
		// No finite travel time (NaN coordinates): walk from point 0 rather
		// than from the search's "none" marker.
		last = idxMin < p.nIf ? idxMin : 0U;
	}
	const float* m1 = p.medium1 + static_cast<size_t>(elem) * p.nIf;
	for (unsigned row = r0 + 1U; row < p.nrows; ++row) {
		const float px = g[row].x, pz = g[row].y;
		auto tc2 = [&](unsigned i) {
			const float2 q = p.ifXZ[i];
			return __fadd_rn(m1[i], hypot_rn(__fsub_rn(px, q.x), __fsub_rn(pz, q.y)));
		};
		unsigned idxMin = last;
		float tMin = tc2(idxMin);
		for (unsigned i = idxMin + 1U; i < p.nIf; ++i) {
			const float tt = tc2(i);
			if (tt >= tMin) break;
			tMin = tt;
			idxMin = i;
		}
		if (idxMin == last) {
			for (int i = static_cast<int>(idxMin) - 1; i >= 0; --i) {
				const float tt = tc2(static_cast<unsigned>(i));
				if (tt >= tMin) break;
				tMin = tt;
				idxMin = static_cast<unsigned>(i);
			}
		}
		out[row * rs] = __fmul_rn(tMin, p.fsInvC2);
		last = idxMin;
	}
}

constexpr unsigned kTmTxShared = 32;   // transmit offsets per step kept in shared memory (per warp)

// v0 + k (v1 - v0) at `position` (0 outside [0, L - 2]), times invScale for
// FP16/BF16 storage.
template<int S>
__device__ __forceinline__ float2 interp(const typename Complex<S>::T* row, float position, unsigned maxPos, float invScale)
{
	float k;
	const int i = split_delay(position, k);
	if (static_cast<unsigned>(i) > maxPos) return make_float2(0.f, 0.f);
	const float2 v0 = Complex<S>::load(row + i);
	const float2 v1 = Complex<S>::load(row + i + 1);
	float2 v = make_float2(__fadd_rn(v0.x, __fmul_rn(k, __fsub_rn(v1.x, v0.x))),
	                       __fadd_rn(v0.y, __fmul_rn(k, __fsub_rn(v1.y, v0.y))));
	if (S != usgb::STORE_F32) v = make_float2(__fmul_rn(v.x, invScale), __fmul_rn(v.y, invScale));
	return v;
}

// One step's contribution at one grid point: the apodized sum over the
// receive elements (each the sum over the step's transmit elements, or the
// single transmit element's term), weighted by the coherence factor of the
// receive terms. ONE_TX: ProcessColumnWithOneTxElem; else ProcessColumn.
// drow: the point's delay of element 0; element e at drow[e * nr].
template<int S, int CF, bool ONE_TX>
__device__ __forceinline__ float2 step_contribution(const TmParams& p, const uint4 st, const float* drow, size_t nr,
		float* txs)
{
	using CT = typename Complex<S>::T;
	const unsigned maxPos = p.L - 2U;
	const float* d = drow + st.y * nr;  // element baseElem + e at d[e * nr]
	const CT* acq = static_cast<const CT*>(p.sig) + st.x * p.acqStride;
	CFState<CF> cf;
	float2 sum = make_float2(0.f, 0.f);
	if (ONE_TX) {
		const float txOffset = __fadd_rn(p.signalOffset, d[st.z * nr]);
		for (unsigned rx = 0; rx < p.numElements; ++rx) {
			const float2 term = interp<S>(acq + rx * p.sigStride, __fadd_rn(txOffset, d[rx * nr]), maxPos, p.invScale);
			const float a = __ldg(&p.apod[rx]);
			sum.x = __fadd_rn(sum.x, __fmul_rn(term.x, a));
			sum.y = __fadd_rn(sum.y, __fmul_rn(term.y, a));
			cf.add(term);
		}
	} else {
		// The step's transmit offsets once, in this warp's shared table (lane
		// fastest: no bank conflicts), when there are at most kTmTxShared.
		const unsigned ntx = st.w - st.z + 1U;
		const bool shared = ntx <= kTmTxShared;
		if (shared) {
			for (unsigned tx = 0; tx < ntx; ++tx) txs[tx * 32U] = __fadd_rn(p.signalOffset, d[(st.z + tx) * nr]);
		}
		for (unsigned rx = 0; rx < p.numElements; ++rx) {
			const float rxDelay = d[rx * nr];
			float2 acc = make_float2(0.f, 0.f);
			const CT* sigRx = acq + rx * p.sigStride;
#pragma unroll 4
			for (unsigned tx = st.z; tx <= st.w; ++tx) {
				const float txOffset = shared ? txs[(tx - st.z) * 32U] : __fadd_rn(p.signalOffset, d[tx * nr]);
				const float2 term = interp<S>(sigRx + (tx - st.z) * p.txStride, __fadd_rn(txOffset, rxDelay), maxPos,
						p.invScale);
				acc.x = __fadd_rn(acc.x, term.x);
				acc.y = __fadd_rn(acc.y, term.y);
			}
			const float a = __ldg(&p.apod[rx]);
			sum.x = __fadd_rn(sum.x, __fmul_rn(acc.x, a));
			sum.y = __fadd_rn(sum.y, __fmul_rn(acc.y, a));
			cf.add(acc);
		}
	}
	if (CF != usgb::CF_NONE) {
		const float f = cf.result(p.numElements, p, sum);
		return make_float2(__fmul_rn(sum.x, f), __fmul_rn(sum.y, f));
	}
	return sum;
}

// A block covers kTmCols neighbouring columns of one row (the lanes of a
// warp: the delay-table reads are coalesced and the gathers of a warp fall on
// few sectors) for kTmStepLanes steps at a time (one warp per step); the
// steps' contributions meet in shared memory and are added in step order,
// as the reference adds them.
constexpr unsigned kTmCols = 32;
constexpr unsigned kTmStepLanes = 8;
constexpr int kTmImageThreads = kTmCols * kTmStepLanes;

template<int S, int CF, bool ONE_TX>
__global__ void __launch_bounds__(kTmImageThreads, 4) tm_image_kernel(const __grid_constant__ TmParams p)
{
	__shared__ float2 contrib[kTmStepLanes][kTmCols];
	__shared__ float txShared[kTmStepLanes][kTmTxShared * kTmCols];
	const unsigned lane = threadIdx.x % kTmCols, sl = threadIdx.x / kTmCols;
	const unsigned col = blockIdx.x * kTmCols + lane;
	const unsigned row = blockIdx.y;
	const bool inGrid = col < p.ncols;
	const bool active = inGrid && row >= p.minRow[col];
	const size_t es = p.ncols;   // table element stride
	const float* drow = p.delay + static_cast<size_t>(row) * p.mux * es + col;
	float2 v = make_float2(0.f, 0.f);
	for (unsigned s0 = 0; s0 < p.numSteps; s0 += kTmStepLanes) {
		const unsigned s = s0 + sl;
		float2 c = make_float2(0.f, 0.f);
		if (active && s < p.numSteps) c = step_contribution<S, CF, ONE_TX>(p, p.steps[s], drow, es, &txShared[sl][lane]);
		contrib[sl][lane] = c;
		__syncthreads();
		if (sl == 0 && active) {
			const unsigned n = min(kTmStepLanes, p.numSteps - s0);
			for (unsigned k = 0; k < n; ++k) {
				v.x = __fadd_rn(v.x, contrib[k][lane].x);
				v.y = __fadd_rn(v.y, contrib[k][lane].y);
			}
		}
		__syncthreads();
	}
	if (sl == 0 && inGrid) p.out[static_cast<size_t>(col) * p.nrows + row] = active ? v : make_float2(0.f, 0.f);
}

template<int S, int CF>
cudaError_t launch_image_cf(const TmParams& p, bool oneTx, cudaStream_t st)
{
	const dim3 grid((p.ncols + kTmCols - 1) / kTmCols, p.nrows);
	if (oneTx) {
		tm_image_kernel<S, CF, true><<<grid, kTmImageThreads, 0, st>>>(p);
	} else {
		tm_image_kernel<S, CF, false><<<grid, kTmImageThreads, 0, st>>>(p);
	}
	return cudaGetLastError();
}

template<int S>
cudaError_t launch_image_s(const TmParams& p, int cf, bool oneTx, cudaStream_t st)
{
	switch (cf) {
	case usgb::CF_PCF: return launch_image_cf<S, usgb::CF_PCF>(p, oneTx, st);
	case usgb::CF_SCF: return launch_image_cf<S, usgb::CF_SCF>(p, oneTx, st);
	case usgb::CF_MF: return launch_image_cf<S, usgb::CF_MF>(p, oneTx, st);
	default: return launch_image_cf<S, usgb::CF_NONE>(p, oneTx, st);
	}
}

cudaError_t launch_image(const TmParams& p, int storage, int cf, bool oneTx, cudaStream_t st)
{
	switch (storage) {
	case usgb::STORE_F16: return launch_image_s<usgb::STORE_F16>(p, cf, oneTx, st);
	case usgb::STORE_BF16: return launch_image_s<usgb::STORE_BF16>(p, cf, oneTx, st);
	default: return launch_image_s<usgb::STORE_F32>(p, cf, oneTx, st);
	}
}

struct Failure {
	int code;
	std::string msg;
};

#define TM_FAIL(CODE, STREAM_EXPR)              \
	do {                                        \
		std::ostringstream os_;                 \
		os_ << STREAM_EXPR;                     \
		throw Failure{(CODE), os_.str()};       \
	} while (0)

#define TM_CUDA(CALL)                                                                          \
	do {                                                                                       \
		const cudaError_t e_ = (CALL);                                                         \
		if (e_ != cudaSuccess) {                                                               \
			TM_FAIL(e_ == cudaErrorMemoryAllocation ? USGB_ERR_OUT_OF_MEMORY : USGB_ERR_CUDA,   \
					#CALL << ": " << cudaGetErrorString(e_));                                  \
		}                                                                                      \
	} while (0)

thread_local std::string g_tmCreateError;

// A device buffer that grows to the largest size asked for.
template<typename T>
struct DevBuf {
	T* ptr = nullptr;
	size_t cap = 0;
	void ensure(size_t n)
	{
		if (n <= cap) return;
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
		TM_CUDA(cudaMalloc(&ptr, std::max<size_t>(n, 1) * sizeof(T)));
		cap = n;
	}
	~DevBuf() { if (ptr) cudaFree(ptr); }
};

}  // namespace

struct usgb_two_medium {
	usgb_two_medium_params prm{};
	unsigned L = 0, U = 1, tapsPerPhase = 1, tapsStride = 4, sigStride = 0;
	usgb::host::FFTTables fft;
	bool stageTw = true;
	size_t elemBytes = 0, rfFloats = 0, sigBytes = 0;
	float scale = 1, pcfFactor = 0, signalOffset = 0;
	float* d_polyTaps = nullptr;
	std::vector<float> polyHost;   // the same taps, for the launch parameters
	float2* d_tw = nullptr;
	float4* d_hilb = nullptr;
	float2* d_stw = nullptr;
	void* d_sig = nullptr;
	DevBuf<float> rf, grid, iface, apod, medium1, delay, value;
	DevBuf<unsigned> minRow;
	DevBuf<uint4> steps;
	std::vector<uint4> hSteps;
	cudaStream_t stream = nullptr;
	bool ownStream = false;
	std::string err;

	~usgb_two_medium()
	{
		if (stream) cudaStreamSynchronize(stream);
		void* dev[] = {d_polyTaps, d_tw, d_hilb, d_stw, d_sig};
		for (void* q : dev) if (q) cudaFree(q);
		if (ownStream && stream) cudaStreamDestroy(stream);
	}
};

namespace {

template<typename F>
int guarded(usgb_two_medium* c, F&& f)
{
	if (!c) return USGB_ERR_INVALID_PARAMETER;
	try {
		f();
		return USGB_OK;
	} catch (const Failure& e) {
		c->err = e.msg;
		return e.code;
	} catch (const std::bad_alloc&) {
		c->err = "host allocation failed";
		return USGB_ERR_OUT_OF_MEMORY;
	} catch (const std::exception& e) {
		c->err = e.what();
		return USGB_ERR_INVALID_STATE;
	}
}

void check_and_derive(usgb_two_medium* c, const usgb_two_medium_params* p)
{
	if (!p) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "null parameters");
	if (p->num_elements == 0 || p->num_elements_mux == 0) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of elements is zero.");
	if (p->num_elements_mux > 1024) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "More than 1024 elements.");
	if (p->num_elements > p->num_elements_mux) {
		TM_FAIL(USGB_ERR_INVALID_PARAMETER, "num_elements (" << p->num_elements << ") > num_elements_mux ("
				<< p->num_elements_mux << ").");
	}
	if (p->num_samples < 2) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of samples (" << p->num_samples << ") is < 2.");
	if (p->num_acquisitions == 0 || p->num_tx == 0) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "No acquisition data.");
	if (p->upsampling == 0 || p->upsampling > 64) {
		TM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid upsampling factor: " << p->upsampling << ". Must be >= 1 and <= 64.");
	}
	if (!(p->pitch > 0) || !(p->center_frequency > 0) || !(p->propagation_speed_1 > 0) || !(p->propagation_speed_2 > 0) ||
			!(p->sampling_frequency > 0)) {
		TM_FAIL(USGB_ERR_INVALID_VALUE, "Pitch, frequencies and propagation speeds must be > 0.");
	}
	if (!(p->max_fermat_block_size >= 0)) TM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid max_fermat_block_size.");
	if (p->coherence > USGB_CF_MF) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid coherence factor method: " << p->coherence << '.');
	if (p->coherence == USGB_CF_PCF && !(p->pcf_gamma >= 0 && p->pcf_gamma <= 100)) {
		TM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid phase_coherence_factor_gamma: " << p->pcf_gamma << '.');
	}
	if (p->storage > USGB_STORE_BF16) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid storage type: " << p->storage << '.');
	c->prm = *p;
	c->U = p->upsampling;
	const unsigned long long L = static_cast<unsigned long long>(p->num_samples) * c->U;
	if (L > (1ULL << 20)) {
		TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of input samples (" << L << ") is greater than " << (1U << 20) << '.');
	}
	c->L = static_cast<unsigned>(L);
	// signalOffset_ (VectorialCombinedTwoMediumImagingProcessor.h:207).
	const float fsUp = p->sampling_frequency * c->U;
	c->signalOffset = fsUp * (p->peak_offset / p->center_frequency) - static_cast<float>(p->signal_start_offset * c->U);
	const float sigma0 = static_cast<float>(usgb::host::kPi / std::sqrt(3.0));
	c->pcfFactor = p->pcf_gamma / sigma0;
	c->scale = (p->storage == USGB_STORE_F32 || p->storage_scale == 0.0f) ? 1.0f : p->storage_scale;
	c->elemBytes = 2 * (p->storage == USGB_STORE_F32 ? 4 : 2);
	c->sigStride = (c->L + 7U) & ~7U;
	c->rfFloats = static_cast<size_t>(p->num_acquisitions) * p->num_tx * p->num_elements * p->num_samples;
	c->sigBytes = static_cast<size_t>(p->num_acquisitions) * p->num_tx * p->num_elements * c->sigStride * c->elemBytes + 256;
}

usgb::PrepParams prep_params(const usgb_two_medium* c, const float* d_rf)
{
	usgb::PrepParams pp{};
	pp.rf = d_rf;
	pp.out = c->d_sig;
	pp.outStride = c->sigStride;
	pp.numSignals = c->prm.num_acquisitions * c->prm.num_tx * c->prm.num_elements;
	pp.ns = c->prm.num_samples;
	pp.U = c->U;
	pp.L = c->L;
	pp.tapsPerPhase = c->tapsPerPhase;
	pp.tapsStride = c->tapsStride;
	pp.polyTaps = c->d_polyTaps;
	usgb::host::set_param_taps(pp, c->polyHost);
	pp.deadZone = 0;  // Util::removeDC(signal, size): the mean of the whole A-scan
	pp.outScale = c->scale;
	usgb::host::set_fft_params(pp, c->fft);
	pp.tw = c->d_tw;
	pp.hilb = c->d_hilb;
	pp.stw = c->stageTw ? c->d_stw : nullptr;
	return pp;
}

void build_tables(usgb_two_medium* c)
{
	usgb::host::PolyTaps poly;
	if (!usgb::host::make_poly_taps(true, c->U, poly)) {
		TM_FAIL(USGB_ERR_INVALID_STATE, "FIR length is not 2*U*K + 1 for upsampling " << c->U);
	}
	c->tapsPerPhase = poly.tapsPerPhase;
	c->tapsStride = poly.tapsStride;
	c->polyHost = poly.poly;
	auto upload = [](auto** dst, const auto& v) {
		using E = typename std::decay_t<decltype(v)>::value_type;
		TM_CUDA(cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(E)));
		if (!v.empty()) TM_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice));
	};
	upload(&c->d_polyTaps, poly.poly);
	if (!usgb::host::make_fft_tables(c->L, c->fft)) TM_FAIL(USGB_ERR_INVALID_STATE, "FFT size " << c->fft.M << " not supported");
	upload(&c->d_tw, c->fft.tw);
	upload(&c->d_hilb, c->fft.hilb);
	upload(&c->d_stw, c->fft.stageTw);
	int dev = 0, maxSmem = 0;
	TM_CUDA(cudaGetDevice(&dev));
	TM_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
	size_t need = usgb::prep_smem_bytes(prep_params(c, nullptr), true);
	if (need > static_cast<size_t>(maxSmem)) {
		c->stageTw = false;
		need = usgb::prep_smem_bytes(prep_params(c, nullptr), true);
	}
	if (need > static_cast<size_t>(maxSmem)) {
		TM_FAIL(USGB_ERR_UNSUPPORTED, "A-scan too long for on-chip preparation (signal length " << c->L << ").");
	}
	TM_CUDA(cudaMalloc(&c->d_sig, c->sigBytes));
	TM_CUDA(cudaMemset(c->d_sig, 0, c->sigBytes));
}

// Checks the steps like the reference's indexing needs them; true = every
// step transmits from one element.
bool check_steps(const usgb_two_medium* c, const usgb_two_medium_step* steps, uint32_t n)
{
	if (!steps || n == 0) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The list of step configurations is empty.");
	const bool oneTx = steps[0].first_tx_elem == steps[0].last_tx_elem;
	const auto& p = c->prm;
	for (uint32_t i = 0; i < n; ++i) {
		const usgb_two_medium_step& s = steps[i];
		if (s.base_elem_idx >= p.num_acquisitions) {
			TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Step " << i << ": acquisition " << s.base_elem_idx << " >= "
					<< p.num_acquisitions << '.');
		}
		if (static_cast<uint64_t>(s.base_elem) + p.num_elements > p.num_elements_mux) {
			TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Step " << i << ": base element " << s.base_elem << " + "
					<< p.num_elements << " elements > " << p.num_elements_mux << '.');
		}
		if (s.first_tx_elem > s.last_tx_elem || s.last_tx_elem >= p.num_elements) {
			TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Step " << i << ": invalid transmit elements " << s.first_tx_elem << ".."
					<< s.last_tx_elem << '.');
		}
		if (!oneTx && s.last_tx_elem - s.first_tx_elem + 1U > p.num_tx) {
			TM_FAIL(USGB_ERR_INVALID_PARAMETER, "Step " << i << ": " << s.last_tx_elem - s.first_tx_elem + 1U
					<< " transmit elements, the acquisitions hold " << p.num_tx << '.');
		}
	}
	return oneTx;
}

void run(usgb_two_medium* c, const float* d_rf, const usgb_two_medium_step* steps, uint32_t numSteps, const float* d_if,
		uint32_t nIf, const float* d_apod, const float* d_grid, uint32_t ncols, uint32_t nrows, float* d_value)
{
	const bool oneTx = check_steps(c, steps, numSteps);
	if (nIf < 2) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The interface needs at least two points (" << nIf << ").");
	if (ncols == 0 || nrows < 2) TM_FAIL(USGB_ERR_INVALID_VALUE, "The grid needs >= 1 column and >= 2 rows.");
	if (ncols > 65535U) TM_FAIL(USGB_ERR_UNSUPPORTED, "Grids of more than 65535 columns are not supported.");
	const auto& prm = c->prm;
	const size_t npix = static_cast<size_t>(ncols) * nrows;
	const size_t tableSize = npix * prm.num_elements_mux;
	if (static_cast<uint64_t>(ncols) * prm.num_elements_mux > 0xFFFFFFFFull ||
			static_cast<uint64_t>(prm.num_elements_mux) * nIf > 0xFFFFFFFFull) {
		TM_FAIL(USGB_ERR_UNSUPPORTED, "Grid or interface too large.");
	}
	c->hSteps.resize(numSteps);
	for (uint32_t i = 0; i < numSteps; ++i) {
		c->hSteps[i] = make_uint4(steps[i].base_elem_idx, steps[i].base_elem, steps[i].first_tx_elem, steps[i].last_tx_elem);
	}
	c->steps.ensure(numSteps);
	c->minRow.ensure(ncols);
	c->medium1.ensure(static_cast<size_t>(prm.num_elements_mux) * nIf);
	c->delay.ensure(tableSize);
	const cudaStream_t st = c->stream;
	TM_CUDA(cudaMemcpyAsync(c->steps.ptr, c->hSteps.data(), numSteps * sizeof(uint4), cudaMemcpyHostToDevice, st));

	TmParams p;
	std::memset(&p, 0, sizeof(p));
	p.ifXZ = reinterpret_cast<const float2*>(d_if);
	p.nIf = nIf;
	p.grid = reinterpret_cast<const float2*>(d_grid);
	p.ncols = ncols;
	p.nrows = nrows;
	p.mux = prm.num_elements_mux;
	p.pitch = prm.pitch;
	p.lambda2 = prm.propagation_speed_2 / prm.center_frequency;
	p.maxBlockWl = static_cast<unsigned>(prm.max_fermat_block_size);
	p.invC1 = 1.0f / prm.propagation_speed_1;
	p.invC2 = 1.0f / prm.propagation_speed_2;
	p.c2ByC1 = prm.propagation_speed_2 / prm.propagation_speed_1;
	p.fsUp = prm.sampling_frequency * c->U;
	p.fsInvC2 = prm.sampling_frequency * c->U / prm.propagation_speed_2;
	p.minRow = c->minRow.ptr;
	p.medium1 = c->medium1.ptr;
	p.delay = c->delay.ptr;
	p.sig = c->d_sig;
	p.sigStride = c->sigStride;
	p.txStride = static_cast<size_t>(prm.num_elements) * c->sigStride;
	p.acqStride = static_cast<size_t>(prm.num_tx) * p.txStride;
	p.L = c->L;
	p.numElements = prm.num_elements;
	p.steps = c->steps.ptr;
	p.numSteps = numSteps;
	p.apod = d_apod;
	p.signalOffset = c->signalOffset;
	p.invScale = 1.0f / c->scale;
	p.pcfFactor = c->pcfFactor;
	p.scfP = prm.scf_p;
	p.out = reinterpret_cast<float2*>(d_value);

	TM_CUDA(usgb::launch_prep(prep_params(c, d_rf), static_cast<int>(prm.storage), true, st));
	tm_min_row_kernel<<<(ncols + kTmThreads - 1) / kTmThreads, kTmThreads, 0, st>>>(p);
	TM_CUDA(cudaGetLastError());
	const unsigned m1 = prm.num_elements_mux * nIf;
	tm_medium1_kernel<<<(m1 + kTmThreads - 1) / kTmThreads, kTmThreads, 0, st>>>(p);
	TM_CUDA(cudaGetLastError());
	const unsigned nd = ncols * prm.num_elements_mux;
	tm_delay_kernel<<<(nd + kTmThreads - 1) / kTmThreads, kTmThreads, 0, st>>>(p);
	TM_CUDA(cudaGetLastError());
	TM_CUDA(launch_image(p, static_cast<int>(prm.storage), static_cast<int>(prm.coherence), oneTx, st));
}

}  // namespace

extern "C" {

int usgb_two_medium_create(const usgb_two_medium_params* params, usgb_two_medium** out)
{
	if (!out) {
		g_tmCreateError = "null output pointer";
		return USGB_ERR_INVALID_PARAMETER;
	}
	*out = nullptr;
	usgb_two_medium* c = nullptr;
	try {
		c = new usgb_two_medium();
		check_and_derive(c, params);
		TM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
		c->ownStream = true;
		build_tables(c);
		*out = c;
		return USGB_OK;
	} catch (const Failure& e) {
		g_tmCreateError = e.msg;
		delete c;
		return e.code;
	} catch (const std::bad_alloc&) {
		g_tmCreateError = "host allocation failed";
		delete c;
		return USGB_ERR_OUT_OF_MEMORY;
	}
}

void usgb_two_medium_destroy(usgb_two_medium* c)
{
	delete c;
}

const char* usgb_two_medium_last_error(const usgb_two_medium* c)
{
	return c ? c->err.c_str() : g_tmCreateError.c_str();
}

int usgb_two_medium_set_stream(usgb_two_medium* c, void* s)
{
	return guarded(c, [&] {
		TM_CUDA(cudaStreamSynchronize(c->stream));
		if (c->ownStream) TM_CUDA(cudaStreamDestroy(c->stream));
		c->stream = static_cast<cudaStream_t>(s);
		c->ownStream = false;
	});
}

int usgb_two_medium_process_device(usgb_two_medium* c, const float* d_rf, const usgb_two_medium_step* steps,
		uint32_t num_steps, const float* d_interface_xz, uint32_t num_interface, const float* d_rx_apod,
		const float* d_grid_xz, uint32_t ncols, uint32_t nrows, float* d_value)
{
	return guarded(c, [&] {
		if (!d_rf || !d_interface_xz || !d_rx_apod || !d_grid_xz || !d_value) {
			TM_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		}
		run(c, d_rf, steps, num_steps, d_interface_xz, num_interface, d_rx_apod, d_grid_xz, ncols, nrows, d_value);
	});
}

int usgb_two_medium_process(usgb_two_medium* c, const float* rf, const usgb_two_medium_step* steps, uint32_t num_steps,
		const float* interface_xz, uint32_t num_interface, const float* rx_apod, const float* grid_xz, uint32_t ncols,
		uint32_t nrows, float* value)
{
	return guarded(c, [&] {
		if (!rf || !interface_xz || !rx_apod || !grid_xz || !value) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "null host pointer");
		if (num_interface < 2) TM_FAIL(USGB_ERR_INVALID_PARAMETER, "The interface needs at least two points (" << num_interface << ").");
		if (ncols == 0 || nrows < 2) TM_FAIL(USGB_ERR_INVALID_VALUE, "The grid needs >= 1 column and >= 2 rows.");
		const size_t npix = static_cast<size_t>(ncols) * nrows;
		const cudaStream_t st = c->stream;
		c->rf.ensure(c->rfFloats);
		c->iface.ensure(2 * static_cast<size_t>(num_interface));
		c->apod.ensure(c->prm.num_elements);
		c->grid.ensure(2 * npix);
		c->value.ensure(2 * npix);
		TM_CUDA(cudaMemcpyAsync(c->rf.ptr, rf, c->rfFloats * sizeof(float), cudaMemcpyHostToDevice, st));
		TM_CUDA(cudaMemcpyAsync(c->iface.ptr, interface_xz, 2 * num_interface * sizeof(float), cudaMemcpyHostToDevice, st));
		TM_CUDA(cudaMemcpyAsync(c->apod.ptr, rx_apod, c->prm.num_elements * sizeof(float), cudaMemcpyHostToDevice, st));
		TM_CUDA(cudaMemcpyAsync(c->grid.ptr, grid_xz, 2 * npix * sizeof(float), cudaMemcpyHostToDevice, st));
		run(c, c->rf.ptr, steps, num_steps, c->iface.ptr, num_interface, c->apod.ptr, c->grid.ptr, ncols, nrows, c->value.ptr);
		TM_CUDA(cudaMemcpyAsync(value, c->value.ptr, 2 * npix * sizeof(float), cudaMemcpyDeviceToHost, st));
		TM_CUDA(cudaStreamSynchronize(st));
	});
}

int usgb_two_medium_synchronize(usgb_two_medium* c)
{
	return guarded(c, [&] { TM_CUDA(cudaStreamSynchronize(c->stream)); });
}

}  // extern "C"
