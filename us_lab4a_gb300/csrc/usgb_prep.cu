// Signal preparation kernels: A-scan upsampling, DC removal and (analytic
// path) Hilbert analytic signal, one thread block per A-scan, everything in
// shared memory.
//
// Reference stages (per A-scan, src/user/processor/VectorialSTAProcessor.h:212-231):
//   Interpolator::interpolate  src/util/Interpolator.h:113-138  (zero stuffing + FIR,
//                              computed there by FFT overlap-save, src/util/FFTWFilter.h:239-289)
//   Util::removeDC             src/util/Util.h:1009-1018
//   HilbertEnvelope::getAnalyticSignal src/util/HilbertEnvelope.h:227-251
// The real-RF path (src/user/processor/DefaultSTAProcessor.h:141-155) stops
// after removeDC and uses the fixed 4x FIR of src/util/Interpolator4X.h.
//
// GB300 design:
// * The FIR is evaluated directly in polyphase form (the zero-stuffed input
//   has only ceil(taps/U) non-zero products per output), from the A-scan held
//   in shared memory; the same linear convolution as the reference's FFT
//   overlap-save.
// * The N-point real FFT of the zero-padded signal is done as an N/2-point
//   complex FFT of the even/odd-packed samples, in place in shared memory
//   (mixed radix 2/3/4/5, decimation in frequency, output in digit-reversed
//   order). The Hilbert multiplier -i*sgn(k) and the real-FFT split are folded
//   into one pass over digit-reversed pairs (k, M-k), and the inverse is an
//   in-place decimation-in-time FFT that consumes the digit-reversed order and
//   returns the imaginary part y[2n] + i y[2n+1] in natural order.
//   The real part of the analytic signal is the DC-free input itself.
#include <cuda_runtime.h>

#include "usgb_common.cuh"
#include "usgb_internal.h"

namespace usgb {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
	return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b)  // a * conj(b)
{
	return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// Multiply by i * s (s = +1 or -1).
__device__ __forceinline__ float2 cmuli(float2 a, float s) { return make_float2(-s * a.y, s * a.x); }

// In-register DFT of size R; SIGN = -1 forward, +1 backward (unnormalised).
template<int R, int SIGN> struct SmallDFT;

template<int SIGN> struct SmallDFT<2, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		const float2 a = v[0], b = v[1];
		v[0] = cadd(a, b);
		v[1] = csub(a, b);
	}
};
template<int SIGN> struct SmallDFT<3, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		const float s1 = 0.86602540378443864676f * SIGN;
		const float2 t1 = cadd(v[1], v[2]);
		const float2 t2 = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
		const float2 d = csub(v[1], v[2]);
		const float2 t3 = make_float2(-s1 * d.y, s1 * d.x);
		v[0] = cadd(v[0], t1);
		v[1] = cadd(t2, t3);
		v[2] = csub(t2, t3);
	}
};
template<int SIGN> struct SmallDFT<4, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
		const float2 t2 = cadd(v[1], v[3]);
		const float2 t3 = cmuli(csub(v[1], v[3]), static_cast<float>(SIGN));
		v[0] = cadd(t0, t2);
		v[2] = csub(t0, t2);
		v[1] = cadd(t1, t3);
		v[3] = csub(t1, t3);
	}
};
template<int SIGN> struct SmallDFT<5, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
		const float s1 = 0.95105651629515357212f * SIGN, s2 = 0.58778525229247312917f * SIGN;
		const float2 a = v[0];
		const float2 b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]);
		const float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
		const float2 r1 = make_float2(a.x + c1 * b1.x + c2 * b2.x, a.y + c1 * b1.y + c2 * b2.y);
		const float2 r2 = make_float2(a.x + c2 * b1.x + c1 * b2.x, a.y + c2 * b1.y + c1 * b2.y);
		const float2 q1 = make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
		const float2 q2 = make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
		const float2 i1 = make_float2(-q1.y, q1.x), i2 = make_float2(-q2.y, q2.x);
		v[0] = make_float2(a.x + b1.x + b2.x, a.y + b1.y + b2.y);
		v[1] = cadd(r1, i1);
		v[4] = csub(r1, i1);
		v[2] = cadd(r2, i2);
		v[3] = csub(r2, i2);
	}
};

// One in-place stage over `data` (M points), blocks of span Ms, radix R.
// Forward (DIF): DFT_R of the R inputs at stride Ms/R, then twiddle
// W_Ms^(p j). Inverse (DIT, the transpose): conjugate twiddle, then DFT_R.
template<int R, bool INVERSE>
__device__ __forceinline__ void fft_stage(float2* data, const float2* __restrict__ tw, unsigned M, unsigned Ms)
{
	const unsigned sub = Ms / R;
	const unsigned twStride = M / Ms;
	const unsigned nb = M / R;
	for (unsigned b = threadIdx.x; b < nb; b += blockDim.x) {
		const unsigned blk = b / sub;
		const unsigned j = b - blk * sub;
		const unsigned base = blk * Ms + j;
		float2 v[R];
#pragma unroll
		for (int q = 0; q < R; ++q) v[q] = data[base + q * sub];
		if (!INVERSE) {
			SmallDFT<R, -1>::run(v);
#pragma unroll
			for (int q = 1; q < R; ++q) v[q] = cmul(v[q], __ldg(&tw[q * j * twStride]));
		} else {
#pragma unroll
			for (int q = 1; q < R; ++q) v[q] = cmulc(v[q], __ldg(&tw[q * j * twStride]));
			SmallDFT<R, +1>::run(v);
		}
#pragma unroll
		for (int q = 0; q < R; ++q) data[base + q * sub] = v[q];
	}
}

template<bool INVERSE>
__device__ void fft_run(float2* data, const PrepParams& p)
{
	if (!INVERSE) {
		unsigned Ms = p.M;
		for (int s = 0; s < p.numStages; ++s) {
			switch (p.radix[s]) {
			case 2: fft_stage<2, false>(data, p.tw, p.M, Ms); break;
			case 3: fft_stage<3, false>(data, p.tw, p.M, Ms); break;
			case 4: fft_stage<4, false>(data, p.tw, p.M, Ms); break;
			default: fft_stage<5, false>(data, p.tw, p.M, Ms); break;
			}
			Ms /= p.radix[s];
			__syncthreads();
		}
	} else {
		// Spans of the forward stages, replayed in reverse order.
		unsigned spans[kMaxFFTStages];
		unsigned Ms = p.M;
		for (int s = 0; s < p.numStages; ++s) { spans[s] = Ms; Ms /= p.radix[s]; }
		for (int s = p.numStages - 1; s >= 0; --s) {
			switch (p.radix[s]) {
			case 2: fft_stage<2, true>(data, p.tw, p.M, spans[s]); break;
			case 3: fft_stage<3, true>(data, p.tw, p.M, spans[s]); break;
			case 4: fft_stage<4, true>(data, p.tw, p.M, spans[s]); break;
			default: fft_stage<5, true>(data, p.tw, p.M, spans[s]); break;
			}
			__syncthreads();
		}
	}
}

// Upsampled sample n from the halo-padded A-scan in shared memory:
// x[n] = sum_t h[r + tU] * rf[n/U + K - t], r = n mod U (the zero-stuffed
// linear convolution shifted by (taps-1)/2 = U*K).
__device__ __forceinline__ float upsampled(const float* rfs, const float* taps, unsigned n, unsigned U, unsigned nt)
{
	const unsigned b = n / U;
	const unsigned r = n - b * U;
	const float* h = taps + r * nt;
	const float* src = rfs + b + (nt - 1);  // rfs index b + 2K - t, nt = 2K + 1
	float acc = 0.f;
	for (unsigned t = 0; t < nt; ++t) acc = fmaf(h[t], src[-static_cast<int>(t)], acc);
	return acc;
}

__device__ float block_sum(float v, float* red)
{
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if (lane == 0) red[warp] = v;
	__syncthreads();
	const int nw = (blockDim.x + 31) >> 5;
	float t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.f;
	if (warp == 0) {
		for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
		if (lane == 0) red[0] = t;
	}
	__syncthreads();
	const float r = red[0];
	__syncthreads();
	return r;
}

// Loads the A-scan into shared memory with K zeros on each side (and one
// spare zero at the end), and the polyphase taps.
__device__ void load_ascan(const PrepParams& p, const float* __restrict__ rf, float* rfs, float* taps)
{
	const unsigned K = (p.tapsPerPhase - 1) / 2;
	const unsigned total = p.ns + 2 * K + 1;
	for (unsigned i = threadIdx.x; i < total; i += blockDim.x) {
		const int j = static_cast<int>(i) - static_cast<int>(K);
		rfs[i] = (j >= 0 && j < static_cast<int>(p.ns)) ? __ldg(&rf[j]) : 0.f;
	}
	const unsigned ntaps = p.U * p.tapsPerPhase;
	for (unsigned i = threadIdx.x; i < ntaps; i += blockDim.x) taps[i] = __ldg(&p.polyTaps[i]);
	__syncthreads();
}

template<int S>
__global__ void __launch_bounds__(kPrepThreads)
prep_analytic_kernel(PrepParams p)
{
	extern __shared__ __align__(16) unsigned char smem[];
	float2* data = reinterpret_cast<float2*>(smem);
	float* rfs = reinterpret_cast<float*>(data + p.M);
	const unsigned K = (p.tapsPerPhase - 1) / 2;
	float* taps = rfs + (p.ns + 2 * K + 1);
	float* red = taps + p.U * p.tapsPerPhase;

	const unsigned a = blockIdx.x;
	const float* rf = p.rf + static_cast<size_t>(a) * p.ns;
	load_ascan(p, rf, rfs, taps);

	const unsigned L = p.L;
	const unsigned nt = p.tapsPerPhase;
	// 1. Upsampled signal, packed z[n'] = x[2n'] + i x[2n'+1], zero past L.
	float part = 0.f;
	for (unsigned m = threadIdx.x; m < p.M; m += blockDim.x) {
		const unsigned n0 = 2 * m, n1 = 2 * m + 1;
		float x0 = 0.f, x1 = 0.f;
		if (n0 < L) {
			x0 = upsampled(rfs, taps, n0, p.U, nt);
			if (n0 >= p.deadZone) part += x0;
		}
		if (n1 < L) {
			x1 = upsampled(rfs, taps, n1, p.U, nt);
			if (n1 >= p.deadZone) part += x1;
		}
		data[m] = make_float2(x0, x1);
	}
	// 2. DC removal: mean of [deadZone, L) subtracted from all L samples.
	const float mean = block_sum(part, red) / static_cast<float>(L - p.deadZone);
	for (unsigned m = threadIdx.x; m < p.M; m += blockDim.x) {
		float2 v = data[m];
		if (2 * m < L) v.x -= mean;
		if (2 * m + 1 < L) v.y -= mean;
		data[m] = v;
	}
	__syncthreads();

	// 3. Forward FFT (digit-reversed output).
	fft_run<false>(data, p);

	// 4. Hilbert multiplier and real-FFT split, on the pairs (k, M-k):
	//    W[k] = i sin(pi k/M) Z[k] + cos(pi k/M) conj(Z[M-k]), W[0] = 0.
	const unsigned half = p.M / 2;
	for (unsigned k = threadIdx.x; k <= half; k += blockDim.x) {
		if (k == 0) {
			data[__ldg(&p.perm[0])] = make_float2(0.f, 0.f);
		} else if (2 * k == p.M) {
			const unsigned q = __ldg(&p.perm[k]);
			const float2 z = data[q];
			data[q] = make_float2(-z.y, z.x);
		} else {
			const unsigned q1 = __ldg(&p.perm[k]);
			const unsigned q2 = __ldg(&p.perm[p.M - k]);
			const float2 A = data[q1], B = data[q2];
			const float2 cs = __ldg(&p.cs[k]);
			data[q1] = make_float2(cs.x * B.x - cs.y * A.y, cs.y * A.x - cs.x * B.y);
			data[q2] = make_float2(-cs.y * B.y - cs.x * A.x, cs.y * B.x + cs.x * A.y);
		}
	}
	__syncthreads();

	// 5. Inverse FFT (natural-order output w[n'] = M * (y[2n'] + i y[2n'+1])).
	fft_run<true>(data, p);

	// 6. Store (x[n], y[n]) for n < L.
	using CT = typename Complex<S>::T;
	CT* out = reinterpret_cast<CT*>(p.out) + static_cast<size_t>(a) * p.outStride;
	const float invM = 1.0f / static_cast<float>(p.M);
	const float sc = p.outScale;
	for (unsigned m = threadIdx.x; 2 * m < L; m += blockDim.x) {
		const float2 w = data[m];
		const unsigned n0 = 2 * m;
		const float x0 = upsampled(rfs, taps, n0, p.U, nt) - mean;
		out[n0] = Complex<S>::pack(x0 * sc, w.x * invM * sc);
		if (n0 + 1 < L) {
			const float x1 = upsampled(rfs, taps, n0 + 1, p.U, nt) - mean;
			out[n0 + 1] = Complex<S>::pack(x1 * sc, w.y * invM * sc);
		}
	}
}

// Real-RF path: upsampling (fixed 4x FIR) and DC removal only.
template<int S>
__global__ void __launch_bounds__(kPrepThreads)
prep_real_kernel(PrepParams p)
{
	extern __shared__ __align__(16) unsigned char smem[];
	float* rfs = reinterpret_cast<float*>(smem);
	const unsigned K = (p.tapsPerPhase - 1) / 2;
	float* taps = rfs + (p.ns + 2 * K + 1);
	float* red = taps + p.U * p.tapsPerPhase;
	const unsigned a = blockIdx.x;
	load_ascan(p, p.rf + static_cast<size_t>(a) * p.ns, rfs, taps);
	const unsigned L = p.L;
	float part = 0.f;
	for (unsigned n = p.deadZone + threadIdx.x; n < L; n += blockDim.x) {
		part += upsampled(rfs, taps, n, p.U, p.tapsPerPhase);
	}
	const float mean = block_sum(part, red) / static_cast<float>(L - p.deadZone);
	using RT = typename Real<S>::T;
	RT* out = reinterpret_cast<RT*>(p.out) + static_cast<size_t>(a) * p.outStride;
	for (unsigned n = threadIdx.x; n < L; n += blockDim.x) {
		out[n] = Real<S>::pack((upsampled(rfs, taps, n, p.U, p.tapsPerPhase) - mean) * p.outScale);
	}
}

}  // namespace

size_t prep_smem_bytes(const PrepParams& p, bool analytic)
{
	const unsigned K = (p.tapsPerPhase - 1) / 2;
	size_t b = (p.ns + 2 * K + 1) * sizeof(float) + p.U * p.tapsPerPhase * sizeof(float) + 32 * sizeof(float);
	if (analytic) b += static_cast<size_t>(p.M) * sizeof(float2);
	return b;
}

cudaError_t launch_prep(const PrepParams& p, int storage, bool analytic, cudaStream_t stream)
{
	const size_t smem = prep_smem_bytes(p, analytic);
	const dim3 grid(p.numSignals), block(kPrepThreads);
	cudaError_t e = cudaSuccess;
#define USGB_LAUNCH_PREP(KERNEL, S)                                                               \
	do {                                                                                          \
		e = cudaFuncSetAttribute(KERNEL<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
		if (e != cudaSuccess) return e;                                                           \
		KERNEL<S><<<grid, block, smem, stream>>>(p);                                              \
	} while (0)
	if (analytic) {
		switch (storage) {
		case STORE_F16: USGB_LAUNCH_PREP(prep_analytic_kernel, STORE_F16); break;
		case STORE_BF16: USGB_LAUNCH_PREP(prep_analytic_kernel, STORE_BF16); break;
		default: USGB_LAUNCH_PREP(prep_analytic_kernel, STORE_F32); break;
		}
	} else {
		switch (storage) {
		case STORE_F16: USGB_LAUNCH_PREP(prep_real_kernel, STORE_F16); break;
		case STORE_BF16: USGB_LAUNCH_PREP(prep_real_kernel, STORE_BF16); break;
		default: USGB_LAUNCH_PREP(prep_real_kernel, STORE_F32); break;
		}
	}
#undef USGB_LAUNCH_PREP
	return cudaGetLastError();
}

}  // namespace usgb
