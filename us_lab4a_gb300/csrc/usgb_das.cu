// Delay-and-sum kernels: per grid point, tx/rx delays, linearly interpolated
// gather over every tx x rx pair, and the coherence factor over the
// per-receiver sums.
//
// Reference: src/user/processor/VectorialSTAProcessor.h:237-338 (analytic,
// with the 3D delays of src/user/processor/Vectorial3DSTAProcessor.h:208-242)
// and src/user/processor/DefaultSTAProcessor.h:158-223 (real RF, SCF);
// coherence factors src/util/CoherenceFactor.h:217-296.
//
// Delays are rounded exactly like the reference's float arithmetic
// (no FMA contraction, IEEE sqrt): delay = (signalOffset + txDelay) + rxDelay,
// with txDelay = dist * invCT. The sample index is floor(delay) and the
// fraction delay - floor(delay) is exact, so every gather reads the same two
// samples with the same weights as the reference; only the order of the
// floating-point sums differs. A gather is skipped unless 0 <= idx and
// idx + 1 < L (src/user/processor/VectorialSTAProcessor.h:277).
#include <cuda_runtime.h>

#include "usgb_common.cuh"
#include "usgb_das_cf.cuh"
#include "usgb_internal.h"

namespace usgb {

namespace {

constexpr int kDirectThreads = 128;

// floor(d) and d - floor(d) for 0 <= d < 2^23: one add with rounding toward
// -inf against 2^23 puts floor(d) in the mantissa. Every other d lands
// outside [0, 2^23) as an unsigned index, so the range test below rejects it:
// -2^23 <= d < 0 gives a sum in [0, 2^23) (index -2^23..-1), a negative sum
// (d < -2^23, -inf) has its sign bit set (index >= 0xB5000000 after the
// wrap), d >= 2^23, +inf and NaN give indices >= 2^23.
__device__ __forceinline__ int split_delay(float d, float& frac)
{
	const float t = __fadd_rd(d, 8388608.0f);
	frac = d - (t - 8388608.0f);
	return static_cast<int>(__float_as_uint(t) - 0x4B000000u);  // wraps, never overflows
}

template<int S, bool ANALYTIC>
__device__ __forceinline__ constexpr size_t sample_bytes()
{
	return ANALYTIC ? sizeof(typename Complex<S>::T) : sizeof(typename Real<S>::T);
}

// acc += (1-k) s[0] + k s[1] (complex or real taps at `s`).
template<int S, bool ANALYTIC>
__device__ __forceinline__ void gather(const char* s, float k, float2& acc)
{
	const float w0 = 1.0f - k;
	if constexpr (ANALYTIC) {
		using CT = typename Complex<S>::T;
		const float2 s0 = Complex<S>::load(reinterpret_cast<const CT*>(s));
		const float2 s1 = Complex<S>::load(reinterpret_cast<const CT*>(s) + 1);
		acc.x = fmaf(w0, s0.x, acc.x);
		acc.y = fmaf(w0, s0.y, acc.y);
		acc.x = fmaf(k, s1.x, acc.x);
		acc.y = fmaf(k, s1.y, acc.y);
	} else {
		using RT = typename Real<S>::T;
		acc.x = fmaf(w0, Real<S>::load(reinterpret_cast<const RT*>(s)), acc.x);
		acc.x = fmaf(k, Real<S>::load(reinterpret_cast<const RT*>(s) + 1), acc.x);
	}
}

// Plain form: one thread per grid point, gathers straight from global
// memory. Receiver-major loop so that each receiver's sum over transmitters
// is complete before it enters the coherence factor.
template<int S, int CF, bool ANALYTIC>
__global__ void __launch_bounds__(kDirectThreads)
das_direct_kernel(DasParams p)
{
	extern __shared__ float txd[];  // [numTx][blockDim.x]
	const unsigned tid = threadIdx.x;
	const unsigned pix = blockIdx.x * blockDim.x + tid;
	const bool active = pix < p.npix;
	float px = 0.f, py = 0.f, pz = 0.f;
	if (active) {
		px = p.grid[3 * pix];
		py = p.grid[3 * pix + 1];
		pz = p.grid[3 * pix + 2];
	}
	for (unsigned t = 0; t < p.numTx; ++t) {
		const float dist = distance3d_z0(__ldg(&p.txXY[2 * t]), __ldg(&p.txXY[2 * t + 1]), px, py, pz);
		txd[t * blockDim.x + tid] = __fadd_rn(p.signalOffset, __fmul_rn(dist, p.invCT));
	}
	if (!active) return;

	const unsigned lastIdx = p.L - 2;
	const size_t txStride = static_cast<size_t>(p.numRx) * p.sigStride;
	float2 total = make_float2(0.f, 0.f);
	CFState<CF> cf;
	for (unsigned r = 0; r < p.numRx; ++r) {
		const float rxd = __fmul_rn(distance3d_z0(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), px, py, pz), p.invCT);
		// The receiver's terms, transmitter by transmitter, into one
		// accumulator (the order every delay-and-sum kernel of the library uses).
		float2 acc = make_float2(0.f, 0.f);
		const char* rsig = static_cast<const char*>(p.sig) + (static_cast<size_t>(r) * p.sigStride) * sample_bytes<S, ANALYTIC>();
		for (unsigned t = 0; t < p.numTx; ++t) {
			float k;
			const int i = split_delay(__fadd_rn(txd[t * blockDim.x + tid], rxd), k);
			if (static_cast<unsigned>(i) <= lastIdx) {
				gather<S, ANALYTIC>(rsig + (t * txStride + i) * sample_bytes<S, ANALYTIC>(), k, acc);
			}
		}
		const float2 rs = receiver_sum(acc, __ldg(&p.apod[r]) * p.invScale);
		total.x += rs.x;
		total.y += rs.y;
		cf.add(rs);
	}
	const float v = ANALYTIC ? magnitude(total) : total.x;
	p.value[pix] = v * p.valueCoef;
	p.factor[pix] = cf.result(p.numRx, p, total);
}

template<int S, int CF, bool ANALYTIC>
cudaError_t launch_direct(const DasParams& p, cudaStream_t stream)
{
	const size_t smem = static_cast<size_t>(p.numTx) * kDirectThreads * sizeof(float);
	cudaError_t e = cudaFuncSetAttribute(das_direct_kernel<S, CF, ANALYTIC>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
	if (e != cudaSuccess) return e;
	const unsigned blocks = (p.npix + kDirectThreads - 1) / kDirectThreads;
	das_direct_kernel<S, CF, ANALYTIC><<<blocks, kDirectThreads, smem, stream>>>(p);
	return cudaGetLastError();
}

template<int S>
cudaError_t dispatch_cf(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	if (!analytic) {
		return (cf == CF_SCF) ? launch_direct<S, CF_SCF, false>(p, stream) : launch_direct<S, CF_NONE, false>(p, stream);
	}
	switch (cf) {
	case CF_PCF: return launch_direct<S, CF_PCF, true>(p, stream);
	case CF_SCF: return launch_direct<S, CF_SCF, true>(p, stream);
	case CF_MF: return launch_direct<S, CF_MF, true>(p, stream);
	default: return launch_direct<S, CF_NONE, true>(p, stream);
	}
}

}  // namespace

cudaError_t launch_das(const DasParams& p, int storage, int cf, bool analytic, int variant, cudaStream_t stream)
{
	if (variant == 1) return launch_das_staged(p, storage, cf, analytic, stream);
	if (variant >= 2 && variant <= 4) return launch_das_group(p, storage, cf, analytic, stream);
	switch (storage) {
	case STORE_F16: return dispatch_cf<STORE_F16>(p, cf, analytic, stream);
	case STORE_BF16: return dispatch_cf<STORE_BF16>(p, cf, analytic, stream);
	default: return dispatch_cf<STORE_F32>(p, cf, analytic, stream);
	}
}

}  // namespace usgb
