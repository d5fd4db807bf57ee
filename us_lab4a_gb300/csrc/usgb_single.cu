// Single-term 3D processors: T1R1 SAFT, TnRn (one focused or diverging
// transmit) and the synthetic-y TnRn array. Each grid point sums one linearly
// interpolated sample per prepared A-scan:
//   Vectorial3DT1R1SAFTProcessor<float>   src/user/processor/Vectorial3DT1R1SAFTProcessor.h:128-236
//   Vectorial3DTnRnProcessor<float>       src/user/processor/Vectorial3DTnRnProcessor.h:163-282
//   SynthYVectorial3DTnRnProcessor<float> src/user/processor/SynthYVectorial3DTnRnProcessor.h:169-305
// The A-scans go through the STA preparation kernel (upsampling, DC removal,
// analytic signal); the delay-and-sum is one thread per grid point with the
// signals read through L1/L2 (one term per signal and point gives no reuse
// across transmit events for a shared-memory stage to exploit).
//
// Every delay and every term is rounded as the reference's float arithmetic
// rounds it (no contraction, IEEE division and square root), so each term
// reads the same two samples with the same weights and equals the
// reference's term bit for bit for FP32 storage; the terms are summed in the
// reference's order (acquisition-major, then signal).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
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
using usgb::distance3d_z0;
using usgb::magnitude;

constexpr int kSingleThreads = 256;
constexpr unsigned kMaxWindow = 256;    // acquisitions of one synthetic-y window
constexpr unsigned kMaxSignals = 1024;  // numElementsMux limit of the reference's configurations

struct SingleParams {
	const void* sig;             // slots x numSignals x sigStride samples (storage type)
	size_t sigStride;            // samples per A-scan
	size_t slotStride;           // samples per acquisition slot
	unsigned L;                  // valid samples per A-scan
	unsigned numSignals;
	const float2* txXY;          // T1R1: numSignals; TnRn: [0] = first element of the group
	const float2* rxXY;          // numSignals
	const float* apod;           // TnRn: numSignals
	const float* grid;           // npix (x, y, z), point (col, row) at col * nrows + row
	unsigned npix, ncols, nrows;
	unsigned tileCols;           // grid columns across a warp (32, 8 or 1)
	float fsUp;                  // fs * U
	float invCT;                 // fs * U / c
	float signalOffset;          // fs * U * peakOffset / fc
	float focusX, focusY, focusZ;
	float firstTxDelay;          // txDelays[0], s
	float valueFactor;           // synthetic y: 1 / window size (as float(1.0 / n)); else 1
	float valueCoef;             // 1 / numSignals
	float invScale;              // 1 / storage scale
	float pcfFactor;
	float scfP;
	float* value;
	float* factor;
	unsigned firstSlot, numSlots, numAcq;
	float yOffset[kMaxWindow];   // per window acquisition: y - centerY (0 outside synthetic y)
};

// floor(d) and d - floor(d) for 0 <= d < 2^23 (one add rounding toward -inf
// against 2^23); every other d, including negatives, infinities and NaN,
// gives an index outside [0, 2^23), which the caller's unsigned range test
// rejects.
__device__ __forceinline__ int split_delay(float d, float& frac)
{
	const float t = __fadd_rd(d, 8388608.0f);
	frac = d - (t - 8388608.0f);
	return static_cast<int>(__float_as_uint(t) - 0x4B000000u);
}

// Geometry::distance3D (src/util/Geometry.h:67-75), rounded as the reference.
__device__ __forceinline__ float distance3d(float x0, float y0, float z0, float x1, float y1, float z1)
{
	const float dx = __fsub_rn(x1, x0);
	const float dy = __fsub_rn(y1, y0);
	const float dz = __fsub_rn(z1, z0);
	return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

// atan2(y, x) for the phase of each single term: octant reduction to
// t = min(|x|, |y|) / max(|x|, |y|) in [0, 1], atan(t) = t P(t^2) with a
// degree-7 polynomial P fitted by weighted least squares on Chebyshev nodes
// (iterated toward the minimax fit), then the octant and sign of (x, y):
// pi / 2 - r above the diagonal, pi - r for x < 0 (and x = -0), the sign of y.
// Largest error over [0, 1] evaluated in FP32: 1.6e-7 rad (about one FP32 ulp
// of pi / 4); the phases only enter standard deviations that are compared
// to 1e-3. Ratios of very small terms are scaled by 2^64 first (exact) so
// that the fast reciprocal sees a normal divisor.
__device__ __forceinline__ float phase_atan2(float y, float x)
{
	const float ax = fabsf(x), ay = fabsf(y);
	float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
	if (mx < 0x1p-64f) {
		mx *= 0x1p64f;
		mn *= 0x1p64f;
	}
	const float t = (mx > 0.f) ? __fdividef(mn, mx) : 0.f;
	const float z = t * t;
	float q = -0.0047803944908082485f;
	q = fmaf(q, z, 0.02455691248178482f);
	q = fmaf(q, z, -0.05990442633628845f);
	q = fmaf(q, z, 0.09942739456892014f);
	q = fmaf(q, z, -0.1402941346168518f);
	q = fmaf(q, z, 0.19971373677253723f);
	q = fmaf(q, z, -0.3333209455013275f);
	q = fmaf(q, z, 0.9999999403953552f);
	float r = q * t;
	if (ay > ax) r = 1.57079632679489662f - r;
	if (signbit(x)) r = 3.14159265358979324f - r;
	return copysignf(r, y);
}

// Phase coherence factor over single terms (src/util/CoherenceFactor.h:267-286:
// population standard deviations of the phases phi and phi -+ pi). One
// update per term, so the sums are kept shifted by the first term's phases
// (sum d, sum d^2 with d = phi - phi_0), which needs no division per term and
// keeps the cancellation of sum d^2 - (sum d)^2 / N small: the phases lie in
// [-pi, pi], so for N terms the rounding of the sums moves the variance by
// about sqrt(N) * 2^-24 * (2 pi)^2, below 1e-4 of the factor for N <= 2^16.
struct SinglePcf {
	unsigned n = 0;
	float k1 = 0.f, k2 = 0.f, s1 = 0.f, q1 = 0.f, s2 = 0.f, q2 = 0.f;
	__device__ __forceinline__ void add(float2 v)
	{
		const float phi = phase_atan2(v.y, v.x);
		const float pi = 3.14159265358979323846f;
		const float aux = phi + ((phi < 0.f) ? pi : -pi);
		if (n == 0) {
			k1 = phi;
			k2 = aux;
		}
		++n;
		const float d1 = __fsub_rn(phi, k1);
		const float d2 = __fsub_rn(aux, k2);
		s1 = __fadd_rn(s1, d1);
		q1 = __fmaf_rn(d1, d1, q1);
		s2 = __fadd_rn(s2, d2);
		q2 = __fmaf_rn(d2, d2, q2);
	}
	template<class P> __device__ float result(unsigned N, const P& p, float2) const
	{
		const float invN = __frcp_rn(static_cast<float>(N));
		const float m1 = __fmul_rn(s1, invN), m2 = __fmul_rn(s2, invN);
		const float v1 = fmaxf(0.f, __fsub_rn(__fmul_rn(q1, invN), __fmul_rn(m1, m1)));
		const float v2 = fmaxf(0.f, __fsub_rn(__fmul_rn(q2, invN), __fmul_rn(m2, m2)));
		const float sd = fminf(__fsqrt_rn(v1), __fsqrt_rn(v2));
		return fmaxf(0.f, __fsub_rn(1.f, __fmul_rn(p.pcfFactor, sd)));
	}
};

template<int CF> struct SingleCF { using T = CFState<CF>; };
template<> struct SingleCF<usgb::CF_PCF> { using T = SinglePcf; };

// MODE 0: T1R1 with separate tx and rx positions; 1: T1R1 with every tx
// position equal to its rx position (one distance per term); 2: TnRn.
//
// A warp covers tileCols neighbouring grid columns at 32 / tileCols
// consecutive depths: the delays of neighbouring columns at one depth differ
// by a few samples, so a warp's gathers of one signal fall into a few
// sectors, where 32 consecutive depths would spread them over one sector
// each (a depth step is tens of upsampled samples).
template<int S, int CF, int MODE>
__global__ void __launch_bounds__(kSingleThreads)
das_single_kernel(const __grid_constant__ SingleParams p)
{
	const unsigned tileRows = kSingleThreads / p.tileCols;
	const unsigned col = blockIdx.x * p.tileCols + threadIdx.x % p.tileCols;
	const unsigned row = blockIdx.y * tileRows + threadIdx.x / p.tileCols;
	if (col >= p.ncols || row >= p.nrows) return;
	const unsigned pix = col * p.nrows + row;
	using CT = typename Complex<S>::T;
	const float px = p.grid[3 * pix];
	const float py = p.grid[3 * pix + 1];
	const float pz = p.grid[3 * pix + 2];
	const unsigned lastIdx = p.L - 2;

	// Travel time from the first element of the group to the focus and its
	// firing delay, in samples (Vectorial3DTnRnProcessor.h:217-222).
	float t0 = 0.f, d0 = 0.f, t0md0 = 0.f;
	if (MODE == 2) {
		const float2 e = __ldg(&p.txXY[0]);
		t0 = __fmul_rn(distance3d_z0(e.x, e.y, p.focusX, p.focusY, p.focusZ), p.invCT);
		d0 = __fmul_rn(p.firstTxDelay, p.fsUp);
		t0md0 = __fsub_rn(t0, d0);
	}

	float2 total = make_float2(0.f, 0.f);
	typename SingleCF<CF>::T cf;
	for (unsigned a = 0; a < p.numAcq; ++a) {
		unsigned slot = p.firstSlot + a;
		if (slot >= p.numSlots) slot -= p.numSlots;
		const float qy = __fsub_rn(py, p.yOffset[a]);
		const CT* sig = static_cast<const CT*>(p.sig) + slot * p.slotStride;
		float base = p.signalOffset;
		if (MODE == 2) {
			const float t1 = __fmul_rn(distance3d(p.focusX, p.focusY, p.focusZ, px, qy, pz), p.invCT);
			const float txDelay = (p.focusZ > 0.f) ? __fadd_rn(__fadd_rn(t1, t0), d0) : __fsub_rn(t1, t0md0);
			base = __fadd_rn(p.signalOffset, txDelay);
		}
#pragma unroll 4
		for (unsigned s = 0; s < p.numSignals; ++s) {
			const float2 r = __ldg(&p.rxXY[s]);
			const float rxDelay = __fmul_rn(distance3d_z0(r.x, r.y, px, qy, pz), p.invCT);
			float delay;
			if (MODE == 2) {
				delay = __fadd_rn(base, rxDelay);
			} else if (MODE == 1) {
				delay = __fadd_rn(__fadd_rn(base, rxDelay), rxDelay);
			} else {
				const float2 t = __ldg(&p.txXY[s]);
				const float txDelay = __fmul_rn(distance3d_z0(t.x, t.y, px, qy, pz), p.invCT);
				delay = __fadd_rn(__fadd_rn(base, txDelay), rxDelay);
			}
			float k;
			const int i = split_delay(delay, k);
			float2 term = make_float2(0.f, 0.f);
			if (static_cast<unsigned>(i) <= lastIdx) {
				const CT* q = sig + s * p.sigStride + i;
				const float2 s0 = Complex<S>::load(q);
				const float2 s1 = Complex<S>::load(q + 1);
				const float w0 = __fsub_rn(1.0f, k);
				const float re = __fadd_rn(__fmul_rn(w0, s0.x), __fmul_rn(k, s1.x));
				const float im = __fadd_rn(__fmul_rn(w0, s0.y), __fmul_rn(k, s1.y));
				if (MODE == 2) {
					// rxApod[i] * term (a term outside the signal stays +0).
					const float w = __fmul_rn(__ldg(&p.apod[s]), p.invScale);
					term = make_float2(__fmul_rn(re, w), __fmul_rn(im, w));
				} else {
					// term added to the +0 of the cleared list (turns -0 into +0).
					term = make_float2(__fadd_rn(__fmul_rn(re, p.invScale), 0.0f), __fadd_rn(__fmul_rn(im, p.invScale), 0.0f));
				}
			}
			total.x = __fadd_rn(total.x, term.x);
			total.y = __fadd_rn(total.y, term.y);
			cf.add(term);
		}
	}
	const float v = __fmul_rn(p.valueFactor, magnitude(total));
	p.value[pix] = __fmul_rn(v, p.valueCoef);
	p.factor[pix] = cf.result(p.numAcq * p.numSignals, p, total);
}

template<int S, int CF>
cudaError_t launch_mode(const SingleParams& p, int mode, cudaStream_t st)
{
	const unsigned tileRows = kSingleThreads / p.tileCols;
	const dim3 blocks((p.ncols + p.tileCols - 1) / p.tileCols, (p.nrows + tileRows - 1) / tileRows);
	switch (mode) {
	case 0: das_single_kernel<S, CF, 0><<<blocks, kSingleThreads, 0, st>>>(p); break;
	case 1: das_single_kernel<S, CF, 1><<<blocks, kSingleThreads, 0, st>>>(p); break;
	default: das_single_kernel<S, CF, 2><<<blocks, kSingleThreads, 0, st>>>(p); break;
	}
	return cudaGetLastError();
}

template<int S>
cudaError_t launch_cf(const SingleParams& p, int cf, int mode, cudaStream_t st)
{
	switch (cf) {
	case usgb::CF_PCF: return launch_mode<S, usgb::CF_PCF>(p, mode, st);
	case usgb::CF_SCF: return launch_mode<S, usgb::CF_SCF>(p, mode, st);
	case usgb::CF_MF: return launch_mode<S, usgb::CF_MF>(p, mode, st);
	default: return launch_mode<S, usgb::CF_NONE>(p, mode, st);
	}
}

cudaError_t launch_single(const SingleParams& p, int storage, int cf, int mode, cudaStream_t st)
{
	switch (storage) {
	case usgb::STORE_F16: return launch_cf<usgb::STORE_F16>(p, cf, mode, st);
	case usgb::STORE_BF16: return launch_cf<usgb::STORE_BF16>(p, cf, mode, st);
	default: return launch_cf<usgb::STORE_F32>(p, cf, mode, st);
	}
}

struct Failure {
	int code;
	std::string msg;
};

#define SINGLE_FAIL(CODE, STREAM_EXPR)          \
	do {                                        \
		std::ostringstream os_;                 \
		os_ << STREAM_EXPR;                     \
		throw Failure{(CODE), os_.str()};       \
	} while (0)

#define SINGLE_CUDA(CALL)                                                                      \
	do {                                                                                       \
		const cudaError_t e_ = (CALL);                                                         \
		if (e_ != cudaSuccess) {                                                               \
			SINGLE_FAIL(e_ == cudaErrorMemoryAllocation ? USGB_ERR_OUT_OF_MEMORY : USGB_ERR_CUDA, \
					#CALL << ": " << cudaGetErrorString(e_));                                  \
		}                                                                                      \
	} while (0)

thread_local std::string g_singleCreateError;

}  // namespace

struct usgb_single {
	usgb_single_params prm{};
	std::vector<float> txXY, rxXY, apod;
	int kernelMode = 0;           // das_single_kernel MODE
	unsigned L = 0, U = 1, deadZone = 0, tapsPerPhase = 1, tapsStride = 4;
	usgb::host::FFTTables fft;
	bool stageTw = true;
	unsigned sigStride = 0;
	size_t slotStride = 0, elemBytes = 0;
	float fsUp = 0, invCT = 0, signalOffset = 0, valueCoef = 0, pcfFactor = 0, scale = 1;
	// Transmit focus (TnRn modes).
	bool txSet = false;
	float focusX = 0, focusY = 0, focusZ = 0, firstTxDelay = 0;
	// Acquisition ring (one slot outside synthetic y).
	unsigned slots = 1;
	uint64_t count = 0;
	std::vector<float> slotY;

	float* d_txXY = nullptr;
	float* d_rxXY = nullptr;
	float* d_apod = nullptr;
	float* d_polyTaps = nullptr;
	std::vector<float> polyHost;   // the same taps, for the launch parameters
	float2* d_tw = nullptr;
	float4* d_hilb = nullptr;
	float2* d_stw = nullptr;
	float* d_rf = nullptr;
	void* d_sig = nullptr;
	float* d_grid = nullptr;
	float* d_value = nullptr;
	float* d_factor = nullptr;
	size_t gridCap = 0;
	unsigned ncols = 0, nrows = 0, npix = 0;
	bool gridSet = false;
	cudaStream_t stream = nullptr;
	bool ownStream = false;
	std::string err;

	~usgb_single()
	{
		if (stream) cudaStreamSynchronize(stream);
		void* dev[] = {d_txXY, d_rxXY, d_apod, d_polyTaps, d_tw, d_hilb, d_stw, d_rf, d_sig, d_grid, d_value,
		               d_factor};
		for (void* p : dev) if (p) cudaFree(p);
		if (ownStream && stream) cudaStreamDestroy(stream);
	}
};

namespace {

template<typename F>
int guarded(usgb_single* c, F&& f)
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

void check_and_derive(usgb_single* c, const usgb_single_params* p)
{
	if (!p) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null parameters");
	if (p->mode > USGB_SINGLE_SYNTH_Y_TNRN) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid processor mode: " << p->mode << '.');
	if (p->num_signals == 0) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of elements is zero.");
	if (p->num_signals > kMaxSignals) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "More than " << kMaxSignals << " elements.");
	if (p->num_samples == 0) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of samples is zero.");
	if (!p->tx_xy || !p->rx_xy) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Missing element positions.");
	const bool tnrn = p->mode != USGB_SINGLE_T1R1_SAFT;
	if (tnrn && !p->rx_apod) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Wrong rx apodization size: 0 (should be " << p->num_signals << ").");
	}
	if (!tnrn && p->rx_apod) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "The T1R1 SAFT processor has no rx apodization.");
	if (p->upsampling == 0 || p->upsampling > 64) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid upsampling factor: " << p->upsampling << ". Must be >= 1 and <= 64.");
	}
	if (!(p->sampling_frequency > 0) || !(p->propagation_speed > 0) || !(p->center_frequency > 0)) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Sampling frequency, propagation speed and center frequency must be > 0.");
	}
	if (!(p->dead_zone_m >= 0)) SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: " << p->dead_zone_m << '.');
	if (p->coherence > USGB_CF_MF) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid coherence factor method: " << p->coherence << '.');
	if (p->coherence == USGB_CF_PCF && !(p->pcf_gamma >= 0 && p->pcf_gamma <= 100)) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid phase_coherence_factor_gamma: " << p->pcf_gamma << '.');
	}
	if (p->coherence == USGB_CF_SCF && !(p->scf_p >= 0 && p->scf_p <= 100)) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid sign_coherence_factor_p: " << p->scf_p << '.');
	}
	if (p->storage > USGB_STORE_BF16) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid storage type: " << p->storage << '.');
	if (p->mode == USGB_SINGLE_SYNTH_Y_TNRN) {
		if (p->max_acquisitions == 0) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "The synthetic-y array needs max_acquisitions >= 1.");
		c->slots = p->max_acquisitions;
	} else if (p->max_acquisitions > 1) {
		SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Only the synthetic-y array keeps more than one acquisition.");
	}

	c->prm = *p;
	c->prm.tx_xy = c->prm.rx_xy = c->prm.rx_apod = nullptr;
	c->U = p->upsampling;
	const unsigned long long L = static_cast<unsigned long long>(p->num_samples) * c->U;
	if (L < 2) SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "The signal length (" << L << ") must be >= 2.");
	if (L > (1ULL << 20)) {
		SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of input samples (" << L << ") is greater than " << (1U << 20) << '.');
	}
	c->L = static_cast<unsigned>(L);
	// deadZoneSamplesUp_ (Vectorial3DT1R1SAFTProcessor.h:106, Vectorial3DTnRnProcessor.h:114).
	const float upFs = c->U * p->sampling_frequency;
	const double dz = upFs * 2.0 * p->dead_zone_m / p->propagation_speed;
	if (!(dz < static_cast<double>(std::numeric_limits<unsigned>::max()))) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: " << p->dead_zone_m << '.');
	}
	c->deadZone = static_cast<unsigned>(dz);
	if (c->deadZone >= c->L) {
		SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: deadZoneSamplesUp_ (" << c->deadZone
				<< ") >= signalLength (" << c->L << ").");
	}
	// signalOffset_ (:117 / :129), invCT (:179 / :211-212).
	c->fsUp = upFs;
	c->invCT = upFs / p->propagation_speed;
	c->signalOffset = upFs * p->peak_offset / p->center_frequency;
	c->valueCoef = 1.0f / static_cast<float>(p->num_signals);
	const float sigma0 = static_cast<float>(usgb::host::kPi / std::sqrt(3.0));
	c->pcfFactor = p->pcf_gamma / sigma0;
	c->scale = (p->storage == USGB_STORE_F32 || p->storage_scale == 0.0f) ? 1.0f : p->storage_scale;

	const unsigned ntx = tnrn ? 1U : p->num_signals;
	c->txXY.assign(p->tx_xy, p->tx_xy + 2 * ntx);
	c->rxXY.assign(p->rx_xy, p->rx_xy + 2 * p->num_signals);
	if (tnrn) {
		c->apod.assign(p->rx_apod, p->rx_apod + p->num_signals);
		c->kernelMode = 2;
	} else {
		c->apod.assign(1, 1.0f);
		c->kernelMode = std::equal(c->txXY.begin(), c->txXY.end(), c->rxXY.begin()) ? 1 : 0;
	}
	c->elemBytes = 2 * (p->storage == USGB_STORE_F32 ? 4 : 2);
	c->sigStride = (c->L + 7U) & ~7U;
	c->slotStride = static_cast<size_t>(p->num_signals) * c->sigStride;
	c->slotY.assign(c->slots, 0.0f);
}

void build_tables(usgb_single* c)
{
	usgb::host::PolyTaps poly;
	if (!usgb::host::make_poly_taps(true, c->U, poly)) {
		SINGLE_FAIL(USGB_ERR_INVALID_STATE, "FIR length is not 2*U*K + 1 for upsampling " << c->U);
	}
	c->tapsPerPhase = poly.tapsPerPhase;
	c->tapsStride = poly.tapsStride;
	c->polyHost = poly.poly;
	auto upload = [](auto** dst, const auto& v) {
		using E = typename std::decay_t<decltype(v)>::value_type;
		SINGLE_CUDA(cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(E)));
		if (!v.empty()) SINGLE_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice));
	};
	upload(&c->d_polyTaps, poly.poly);
	if (!usgb::host::make_fft_tables(c->L, c->fft)) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "FFT size " << c->fft.M << " not supported");
	upload(&c->d_tw, c->fft.tw);
	upload(&c->d_hilb, c->fft.hilb);
	upload(&c->d_stw, c->fft.stageTw);
	upload(&c->d_txXY, c->txXY);
	upload(&c->d_rxXY, c->rxXY);
	upload(&c->d_apod, c->apod);
}

usgb::PrepParams prep_params(const usgb_single* c, const float* d_rf, void* d_out)
{
	usgb::PrepParams pp{};
	pp.rf = d_rf;
	pp.out = d_out;
	pp.outStride = c->sigStride;
	pp.numSignals = c->prm.num_signals;
	pp.ns = c->prm.num_samples;
	pp.U = c->U;
	pp.L = c->L;
	pp.tapsPerPhase = c->tapsPerPhase;
	pp.tapsStride = c->tapsStride;
	pp.polyTaps = c->d_polyTaps;
	usgb::host::set_param_taps(pp, c->polyHost);
	pp.deadZone = c->deadZone;
	pp.outScale = c->scale;
	usgb::host::set_fft_params(pp, c->fft);
	pp.tw = c->d_tw;
	pp.hilb = c->d_hilb;
	pp.stw = c->stageTw ? c->d_stw : nullptr;
	return pp;
}

void check_prep_fits(usgb_single* c)
{
	int dev = 0, maxSmem = 0;
	SINGLE_CUDA(cudaGetDevice(&dev));
	SINGLE_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
	size_t need = usgb::prep_smem_bytes(prep_params(c, nullptr, nullptr), true);
	if (need > static_cast<size_t>(maxSmem)) {
		c->stageTw = false;
		need = usgb::prep_smem_bytes(prep_params(c, nullptr, nullptr), true);
	}
	if (need > static_cast<size_t>(maxSmem)) {
		SINGLE_FAIL(USGB_ERR_UNSUPPORTED, "A-scan too long for on-chip preparation: needs " << need
				<< " bytes of shared memory, the device offers " << maxSmem << " (signal length " << c->L << ").");
	}
}

void alloc_buffers(usgb_single* c)
{
	const size_t rfBytes = static_cast<size_t>(c->prm.num_signals) * c->prm.num_samples * sizeof(float);
	SINGLE_CUDA(cudaMalloc(&c->d_rf, rfBytes));
	const size_t sigBytes = c->slots * c->slotStride * c->elemBytes + 256;
	SINGLE_CUDA(cudaMalloc(&c->d_sig, sigBytes));
	SINGLE_CUDA(cudaMemset(c->d_sig, 0, sigBytes));
}

void ensure_grid(usgb_single* c, uint32_t ncols, uint32_t nrows)
{
	if (ncols == 0) SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Zero columns in the grid.");
	if (nrows == 0) SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Zero rows in the grid.");
	const size_t npix = static_cast<size_t>(ncols) * nrows;
	if (npix > (1ULL << 31)) SINGLE_FAIL(USGB_ERR_INVALID_VALUE, "Grid too large.");
	if (npix > c->gridCap) {
		SINGLE_CUDA(cudaStreamSynchronize(c->stream));
		if (c->d_grid) { cudaFree(c->d_grid); c->d_grid = nullptr; }
		if (c->d_value) { cudaFree(c->d_value); c->d_value = nullptr; }
		if (c->d_factor) { cudaFree(c->d_factor); c->d_factor = nullptr; }
		c->gridCap = 0;
		SINGLE_CUDA(cudaMalloc(&c->d_grid, npix * 3 * sizeof(float)));
		SINGLE_CUDA(cudaMalloc(&c->d_value, npix * sizeof(float)));
		SINGLE_CUDA(cudaMalloc(&c->d_factor, npix * sizeof(float)));
		c->gridCap = npix;
	}
	c->ncols = ncols;
	c->nrows = nrows;
	c->npix = static_cast<unsigned>(npix);
}

void check_tx(const usgb_single* c)
{
	if (c->prm.mode != USGB_SINGLE_T1R1_SAFT && !c->txSet) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "Empty tx delay list.");
}

// Prepares one acquisition into its ring slot.
void prepare_acquisition(usgb_single* c, const float* d_rf, unsigned slot)
{
	void* out = static_cast<char*>(c->d_sig) + slot * c->slotStride * c->elemBytes;
	SINGLE_CUDA(usgb::launch_prep(prep_params(c, d_rf, out), static_cast<int>(c->prm.storage), true, c->stream));
}

// Delay-and-sum over acquisitions first..last (ring numbers) into d_value/d_factor.
void run_das(usgb_single* c, uint64_t first, uint64_t last, float* d_value, float* d_factor)
{
	if (!c->gridSet) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
	check_tx(c);
	const unsigned n = static_cast<unsigned>(last - first + 1);
	SingleParams p;
	std::memset(&p, 0, sizeof(p));
	p.sig = c->d_sig;
	p.sigStride = c->sigStride;
	p.slotStride = c->slotStride;
	p.L = c->L;
	p.numSignals = c->prm.num_signals;
	p.txXY = reinterpret_cast<const float2*>(c->d_txXY);
	p.rxXY = reinterpret_cast<const float2*>(c->d_rxXY);
	p.apod = c->d_apod;
	p.grid = c->d_grid;
	p.npix = c->npix;
	p.ncols = c->ncols;
	p.nrows = c->nrows;
	p.tileCols = c->ncols >= 32 ? 32U : (c->ncols >= 8 ? 8U : 1U);
	while (p.tileCols > 1 && (c->nrows + kSingleThreads / p.tileCols - 1) / (kSingleThreads / p.tileCols) > 65535U) {
		p.tileCols = p.tileCols == 32 ? 8U : 1U;
	}
	if ((c->nrows + kSingleThreads - 1) / kSingleThreads > 65535U) {
		SINGLE_FAIL(USGB_ERR_UNSUPPORTED, "Grids of more than " << 65535U * kSingleThreads << " rows are not supported.");
	}
	p.fsUp = c->fsUp;
	p.invCT = c->invCT;
	p.signalOffset = c->signalOffset;
	p.focusX = c->focusX;
	p.focusY = c->focusY;
	p.focusZ = c->focusZ;
	p.firstTxDelay = c->firstTxDelay;
	p.valueCoef = c->valueCoef;
	p.invScale = 1.0f / c->scale;
	p.pcfFactor = c->pcfFactor;
	p.scfP = c->prm.scf_p;
	p.value = d_value;
	p.factor = d_factor;
	p.firstSlot = static_cast<unsigned>(first % c->slots);
	p.numSlots = c->slots;
	p.numAcq = n;
	if (c->prm.mode == USGB_SINGLE_SYNTH_Y_TNRN) {
		// valueFactor = 1.0 / numAcq (double, stored as float); the window's y
		// is relative to acquisition (first + last) / 2 (SynthYVectorial3DTnRnProcessor.h:229-232, 258-259).
		p.valueFactor = static_cast<float>(1.0 / n);
		const float centerY = c->slotY[((first + last) / 2) % c->slots];
		for (unsigned a = 0; a < n; ++a) p.yOffset[a] = c->slotY[(first + a) % c->slots] - centerY;
	} else {
		p.valueFactor = 1.0f;
	}
	SINGLE_CUDA(launch_single(p, static_cast<int>(c->prm.storage), static_cast<int>(c->prm.coherence), c->kernelMode,
			c->stream));
}

void check_window(const usgb_single* c, uint32_t first, uint32_t last)
{
	if (c->prm.mode != USGB_SINGLE_SYNTH_Y_TNRN) {
		SINGLE_FAIL(USGB_ERR_INVALID_STATE, "Acquisition windows belong to the synthetic-y processor.");
	}
	if (first > last) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid acquisition window: " << first << " > " << last << '.');
	if (last >= c->count) {
		SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Acquisition " << last << " has not been added (" << c->count << " so far).");
	}
	if (c->count - first > c->slots) {
		SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "Acquisition " << first << " is no longer on the device (the last "
				<< c->slots << " are kept).");
	}
	if (last - first + 1 > kMaxWindow) {
		SINGLE_FAIL(USGB_ERR_UNSUPPORTED, "Windows of more than " << kMaxWindow << " acquisitions are not supported.");
	}
}

void copy_out(usgb_single* c, float* value, float* factor)
{
	SINGLE_CUDA(cudaMemcpyAsync(value, c->d_value, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
	if (factor) SINGLE_CUDA(cudaMemcpyAsync(factor, c->d_factor, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
	SINGLE_CUDA(cudaStreamSynchronize(c->stream));
}

}  // namespace

extern "C" {

int usgb_single_create(const usgb_single_params* params, usgb_single** out)
{
	if (!out) {
		g_singleCreateError = "null output pointer";
		return USGB_ERR_INVALID_PARAMETER;
	}
	*out = nullptr;
	usgb_single* c = nullptr;
	try {
		c = new usgb_single();
		check_and_derive(c, params);
		SINGLE_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
		c->ownStream = true;
		build_tables(c);
		check_prep_fits(c);
		alloc_buffers(c);
		*out = c;
		return USGB_OK;
	} catch (const Failure& e) {
		g_singleCreateError = e.msg;
		delete c;
		return e.code;
	} catch (const std::bad_alloc&) {
		g_singleCreateError = "host allocation failed";
		delete c;
		return USGB_ERR_OUT_OF_MEMORY;
	}
}

void usgb_single_destroy(usgb_single* c)
{
	delete c;
}

const char* usgb_single_last_error(const usgb_single* c)
{
	return c ? c->err.c_str() : g_singleCreateError.c_str();
}

int usgb_single_set_stream(usgb_single* c, void* s)
{
	return guarded(c, [&] {
		SINGLE_CUDA(cudaStreamSynchronize(c->stream));
		if (c->ownStream) SINGLE_CUDA(cudaStreamDestroy(c->stream));
		c->stream = static_cast<cudaStream_t>(s);
		c->ownStream = false;
	});
}

int usgb_single_set_tx_delays(usgb_single* c, float focus_x, float focus_y, float focus_z, const float* tx_delays,
		uint32_t count)
{
	return guarded(c, [&] {
		if (count == 0 || !tx_delays) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "Empty tx delay list.");
		c->focusX = focus_x;
		c->focusY = focus_y;
		c->focusZ = focus_z;
		c->firstTxDelay = tx_delays[0];
		c->txSet = true;
	});
}

int usgb_single_set_grid(usgb_single* c, const float* xyz, uint32_t ncols, uint32_t nrows)
{
	return guarded(c, [&] {
		if (!xyz) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null grid");
		ensure_grid(c, ncols, nrows);
		SINGLE_CUDA(cudaMemcpyAsync(c->d_grid, xyz, static_cast<size_t>(c->npix) * 3 * sizeof(float),
				cudaMemcpyHostToDevice, c->stream));
		SINGLE_CUDA(cudaStreamSynchronize(c->stream));
		c->gridSet = true;
	});
}

int usgb_single_set_grid_device(usgb_single* c, const float* d_xyz, uint32_t ncols, uint32_t nrows)
{
	return guarded(c, [&] {
		if (!d_xyz) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null grid");
		ensure_grid(c, ncols, nrows);
		SINGLE_CUDA(cudaMemcpyAsync(c->d_grid, d_xyz, static_cast<size_t>(c->npix) * 3 * sizeof(float),
				cudaMemcpyDeviceToDevice, c->stream));
		c->gridSet = true;
	});
}

int usgb_single_process_device(usgb_single* c, const float* d_rf, float* d_value, float* d_factor)
{
	return guarded(c, [&] {
		if (!d_rf || !d_value || !d_factor) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (c->prm.mode == USGB_SINGLE_SYNTH_Y_TNRN) {
			SINGLE_FAIL(USGB_ERR_INVALID_STATE, "The synthetic-y processor forms images of acquisition windows.");
		}
		if (!c->gridSet) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		check_tx(c);
		prepare_acquisition(c, d_rf, 0);
		run_das(c, 0, 0, d_value, d_factor);
	});
}

int usgb_single_process(usgb_single* c, const float* rf, float* value, float* factor)
{
	return guarded(c, [&] {
		if (!rf || !value) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null host pointer");
		if (c->prm.mode == USGB_SINGLE_SYNTH_Y_TNRN) {
			SINGLE_FAIL(USGB_ERR_INVALID_STATE, "The synthetic-y processor forms images of acquisition windows.");
		}
		if (!c->gridSet) SINGLE_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		check_tx(c);
		const size_t rfBytes = static_cast<size_t>(c->prm.num_signals) * c->prm.num_samples * sizeof(float);
		SINGLE_CUDA(cudaMemcpyAsync(c->d_rf, rf, rfBytes, cudaMemcpyHostToDevice, c->stream));
		prepare_acquisition(c, c->d_rf, 0);
		run_das(c, 0, 0, c->d_value, c->d_factor);
		copy_out(c, value, factor);
	});
}

int usgb_single_add_acquisition_device(usgb_single* c, const float* d_rf, float y)
{
	return guarded(c, [&] {
		if (!d_rf) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (c->prm.mode != USGB_SINGLE_SYNTH_Y_TNRN) {
			SINGLE_FAIL(USGB_ERR_INVALID_STATE, "Acquisitions are added to the synthetic-y processor only.");
		}
		const unsigned slot = static_cast<unsigned>(c->count % c->slots);
		prepare_acquisition(c, d_rf, slot);
		c->slotY[slot] = y;
		++c->count;
	});
}

int usgb_single_add_acquisition(usgb_single* c, const float* rf, float y)
{
	return guarded(c, [&] {
		if (!rf) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null host pointer");
		if (c->prm.mode != USGB_SINGLE_SYNTH_Y_TNRN) {
			SINGLE_FAIL(USGB_ERR_INVALID_STATE, "Acquisitions are added to the synthetic-y processor only.");
		}
		const size_t rfBytes = static_cast<size_t>(c->prm.num_signals) * c->prm.num_samples * sizeof(float);
		SINGLE_CUDA(cudaMemcpyAsync(c->d_rf, rf, rfBytes, cudaMemcpyHostToDevice, c->stream));
		const unsigned slot = static_cast<unsigned>(c->count % c->slots);
		prepare_acquisition(c, c->d_rf, slot);
		c->slotY[slot] = y;
		++c->count;
	});
}

int usgb_single_num_acquisitions(const usgb_single* c, uint32_t* count)
{
	if (!c || !count) return USGB_ERR_INVALID_PARAMETER;
	*count = static_cast<uint32_t>(c->count);
	return USGB_OK;
}

int usgb_single_process_window_device(usgb_single* c, uint32_t first_acq, uint32_t last_acq, float* d_value,
		float* d_factor)
{
	return guarded(c, [&] {
		if (!d_value || !d_factor) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		check_window(c, first_acq, last_acq);
		run_das(c, first_acq, last_acq, d_value, d_factor);
	});
}

int usgb_single_process_window(usgb_single* c, uint32_t first_acq, uint32_t last_acq, float* value, float* factor)
{
	return guarded(c, [&] {
		if (!value) SINGLE_FAIL(USGB_ERR_INVALID_PARAMETER, "null host pointer");
		check_window(c, first_acq, last_acq);
		run_das(c, first_acq, last_acq, c->d_value, c->d_factor);
		copy_out(c, value, factor);
	});
}

int usgb_single_synchronize(usgb_single* c)
{
	return guarded(c, [&] { SINGLE_CUDA(cudaStreamSynchronize(c->stream)); });
}

}  // extern "C"
