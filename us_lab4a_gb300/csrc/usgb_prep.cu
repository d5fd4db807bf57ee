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
// * The FIR is evaluated directly in polyphase form: the FIR length is
//   2UK + 1, so output n = bU + r depends on input samples b - K .. b + K
//   only. A thread takes one input position b, keeps its 2K + 1 input samples
//   in registers and produces all U phases from them, with the taps read as
//   broadcast float4 loads from shared memory. This is the same linear
//   convolution the reference computes with an FFT overlap-save filter.
// * The N-point real FFT of the zero-padded signal is done as an N/2-point
//   complex FFT of the even/odd-packed samples, in place in shared memory
//   (mixed radix 2/3/4/5/6/8/9/15/16, decimation in frequency, output in digit-reversed
//   order; the packed buffer read as floats is the signal itself). The
//   Hilbert multiplier -i*sgn(k) and the real-FFT split are folded into one
//   pass over digit-reversed pairs (k, M-k), and the inverse is an in-place
//   decimation-in-time FFT that consumes the digit-reversed order and returns
//   the imaginary part y[n] in natural order. The real part of the analytic
//   signal is the DC-free input itself. Blocks of 512 threads (one an SM)
//   park it in tensor memory (tcgen05.st, each thread in its own lane) before
//   the FFT overwrites it in shared memory and store whole complex samples in
//   one last pass (tcgen05.ld); smaller blocks store the real parts before
//   the FFT and the imaginary parts in the last pass.
// * Butterflies use packed FP32x2 arithmetic for complex sums and for the
//   i-products of the 3-, 4- and 5-point DFTs (each component rounded as the
//   scalar form rounds it).
// * Each butterfly reads one twiddle W_Ms^j and forms its powers in
//   registers: the first stage from a two-level table (W^m = hi[m / 128] *
//   lo[m % 128]), later stages from per-stage tables indexed by j, so that
//   consecutive lanes read consecutive words. Stage indices use
//   multiply-shift division by host-computed constants.
#include <algorithm>

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
// Complex sums as one packed FP32x2 operation each (a - b as fma(b, -1, a):
// the exact difference rounded once, as a subtraction rounds it).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
// Multiply by i * s (s = +1 or -1).
__device__ __forceinline__ float2 cmuli(float2 a, float s) { return make_float2(-s * a.y, s * a.x); }
__device__ __forceinline__ float2 splat(float c) { return make_float2(c, c); }
// (a - b) with its components swapped: (a.y - b.y, a.x - b.x). A product
// i * s * (a - b) = (-s (a.y - b.y), s (a.x - b.x)) then enters a packed
// fma with the sign pair (-s, s), and a +/- i * s * (a - b) is one packed
// fma per output, each component rounded once as the scalar sum rounds it.
__device__ __forceinline__ float2 csub_swapped(float2 a, float2 b) { return make_float2(a.y - b.y, a.x - b.x); }

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
		const float2 t2 = __ffma2_rn(splat(-0.5f), t1, v[0]);
		const float2 ds = csub_swapped(v[1], v[2]);
		v[0] = cadd(v[0], t1);
		v[1] = __ffma2_rn(ds, make_float2(-s1, s1), t2);
		v[2] = __ffma2_rn(ds, make_float2(s1, -s1), t2);
	}
};
template<int SIGN> struct SmallDFT<4, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		constexpr float sg = static_cast<float>(SIGN);
		const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
		const float2 t2 = cadd(v[1], v[3]);
		const float2 ds = csub_swapped(v[1], v[3]);
		v[0] = cadd(t0, t2);
		v[2] = csub(t0, t2);
		v[1] = __ffma2_rn(ds, make_float2(-sg, sg), t1);
		v[3] = __ffma2_rn(ds, make_float2(sg, -sg), t1);
	}
};
template<int SIGN> struct SmallDFT<5, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
		const float s1 = 0.95105651629515357212f * SIGN, s2 = 0.58778525229247312917f * SIGN;
		const float2 a = v[0];
		const float2 b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]);
		const float2 d1 = csub_swapped(v[1], v[4]), d2 = csub_swapped(v[2], v[3]);
		const float2 r1 = __ffma2_rn(splat(c2), b2, __ffma2_rn(splat(c1), b1, a));
		const float2 r2 = __ffma2_rn(splat(c1), b2, __ffma2_rn(splat(c2), b1, a));
		// q1, q2 with swapped components (d1, d2 are swapped).
		const float2 q1 = __ffma2_rn(splat(s2), d2, __fmul2_rn(splat(s1), d1));
		const float2 q2 = __ffma2_rn(splat(-s1), d2, __fmul2_rn(splat(s2), d1));
		const float2 mp = make_float2(-1.0f, 1.0f), pm = make_float2(1.0f, -1.0f);
		v[0] = cadd(cadd(a, b1), b2);
		v[1] = __ffma2_rn(q1, mp, r1);
		v[4] = __ffma2_rn(q1, pm, r1);
		v[2] = __ffma2_rn(q2, mp, r2);
		v[3] = __ffma2_rn(q2, pm, r2);
	}
};

template<int SIGN> struct SmallDFT<8, SIGN> {
	static __device__ __forceinline__ void run(float2* v)
	{
		// Two 4-point DFTs of the even and odd inputs, then X[k] = E[k] +
		// W8^k O[k] and X[k + 4] = E[k] - W8^k O[k], W8 = exp(SIGN 2 pi i / 8).
		float2 e[4] = {v[0], v[2], v[4], v[6]};
		float2 o[4] = {v[1], v[3], v[5], v[7]};
		SmallDFT<4, SIGN>::run(e);
		SmallDFT<4, SIGN>::run(o);
		const float r = 0.70710678118654752440f;
		const float sg = static_cast<float>(SIGN);
		const float2 o1 = make_float2(r * (o[1].x - sg * o[1].y), r * (o[1].y + sg * o[1].x));
		const float2 o2 = cmuli(o[2], sg);
		const float2 o3 = make_float2(r * (-o[3].x - sg * o[3].y), r * (sg * o[3].x - o[3].y));
		v[0] = cadd(e[0], o[0]);
		v[4] = csub(e[0], o[0]);
		v[1] = cadd(e[1], o1);
		v[5] = csub(e[1], o1);
		v[2] = cadd(e[2], o2);
		v[6] = csub(e[2], o2);
		v[3] = cadd(e[3], o3);
		v[7] = csub(e[3], o3);
	}
};

// (cos, sin)(2 pi m / R) for the composite radices (m < R).
template<int R> __device__ __forceinline__ float2 root(int m);
template<> __device__ __forceinline__ float2 root<6>(int m)
{
	switch (m) {
	case 0: return make_float2(1.0f, 0.0f);
	case 1: return make_float2(0.5f, 0.86602540378443864676f);
	case 2: return make_float2(-0.5f, 0.86602540378443864676f);
	case 3: return make_float2(-1.0f, 0.0f);
	case 4: return make_float2(-0.5f, -0.86602540378443864676f);
	default: return make_float2(0.5f, -0.86602540378443864676f);
	}
}
template<> __device__ __forceinline__ float2 root<9>(int m)
{
	switch (m) {
	case 0: return make_float2(1.0f, 0.0f);
	case 1: return make_float2(0.76604444311897803520f, 0.64278760968653932632f);
	case 2: return make_float2(0.17364817766693034885f, 0.98480775301220805936f);
	case 3: return make_float2(-0.5f, 0.86602540378443864676f);
	case 4: return make_float2(-0.93969262078590838405f, 0.34202014332566873304f);
	case 5: return make_float2(-0.93969262078590838405f, -0.34202014332566873304f);
	case 6: return make_float2(-0.5f, -0.86602540378443864676f);
	case 7: return make_float2(0.17364817766693034885f, -0.98480775301220805936f);
	default: return make_float2(0.76604444311897803520f, -0.64278760968653932632f);
	}
}
// exp(2 pi i m / 10), m < 10: angles of 36 degrees.
template<> __device__ __forceinline__ float2 root<10>(int m)
{
	constexpr float c1 = 0.80901699437494742410f, s1 = 0.58778525229247312917f;
	constexpr float c2 = 0.30901699437494742410f, s2 = 0.95105651629515357212f;
	switch (m) {
	case 0: return make_float2(1.0f, 0.0f);
	case 1: return make_float2(c1, s1);
	case 2: return make_float2(c2, s2);
	case 3: return make_float2(-c2, s2);
	case 4: return make_float2(-c1, s1);
	case 5: return make_float2(-1.0f, 0.0f);
	case 6: return make_float2(-c1, -s1);
	case 7: return make_float2(-c2, -s2);
	case 8: return make_float2(c2, -s2);
	default: return make_float2(c1, -s1);
	}
}
// exp(2 pi i m / 12), m < 12: angles of 30 degrees.
template<> __device__ __forceinline__ float2 root<12>(int m)
{
	constexpr float h = 0.86602540378443864676f;
	switch (m) {
	case 0: return make_float2(1.0f, 0.0f);
	case 1: return make_float2(h, 0.5f);
	case 2: return make_float2(0.5f, h);
	case 3: return make_float2(0.0f, 1.0f);
	case 4: return make_float2(-0.5f, h);
	case 5: return make_float2(-h, 0.5f);
	case 6: return make_float2(-1.0f, 0.0f);
	case 7: return make_float2(-h, -0.5f);
	case 8: return make_float2(-0.5f, -h);
	case 9: return make_float2(0.0f, -1.0f);
	case 10: return make_float2(0.5f, -h);
	default: return make_float2(h, -0.5f);
	}
}
// exp(2 pi i m / 15), m < 15: angles of 24 degrees (m > 7: conjugates of 15 - m).
template<> __device__ __forceinline__ float2 root<15>(int m)
{
	const bool lower = m > 7;
	float c, s;
	switch (lower ? 15 - m : m) {
	case 0: c = 1.0f; s = 0.0f; break;
	case 1: c = 0.91354545764260089550f; s = 0.40673664307580020775f; break;
	case 2: c = 0.66913060635885821383f; s = 0.74314482547739423501f; break;
	case 3: c = 0.30901699437494742410f; s = 0.95105651629515357212f; break;
	case 4: c = -0.10452846326765347140f; s = 0.99452189536827333692f; break;
	case 5: c = -0.5f; s = 0.86602540378443864676f; break;
	case 6: c = -0.80901699437494742410f; s = 0.58778525229247312917f; break;
	default: c = -0.97814760073380563793f; s = 0.20791169081775933710f; break;
	}
	return make_float2(c, lower ? -s : s);
}
// exp(2 pi i m / 16), m < 16: angles of 22.5 degrees.
template<> __device__ __forceinline__ float2 root<16>(int m)
{
	constexpr float a = 0.92387953251128675613f, b = 0.38268343236508977173f, h = 0.70710678118654752440f;
	switch (m) {
	case 0: return make_float2(1.0f, 0.0f);
	case 1: return make_float2(a, b);
	case 2: return make_float2(h, h);
	case 3: return make_float2(b, a);
	case 4: return make_float2(0.0f, 1.0f);
	case 5: return make_float2(-b, a);
	case 6: return make_float2(-h, h);
	case 7: return make_float2(-a, b);
	case 8: return make_float2(-1.0f, 0.0f);
	case 9: return make_float2(-a, -b);
	case 10: return make_float2(-h, -h);
	case 11: return make_float2(-b, -a);
	case 12: return make_float2(0.0f, -1.0f);
	case 13: return make_float2(b, -a);
	case 14: return make_float2(h, -h);
	default: return make_float2(a, -b);
	}
}
// DFT of size R = R1 R2 by the two-factor decomposition: input n = R2 n1 +
// n2, output k = k1 + R1 k2; R2 DFTs of size R1, internal twiddles
// W_R^(n2 k1), then R1 DFTs of size R2 (all in registers).
template<int R1, int R2, int SIGN>
__device__ __forceinline__ void composite_dft(float2* v)
{
	constexpr int R = R1 * R2;
	float2 a[R];
#pragma unroll
	for (int n2 = 0; n2 < R2; ++n2) {
		float2 t[R1];
#pragma unroll
		for (int n1 = 0; n1 < R1; ++n1) t[n1] = v[R2 * n1 + n2];
		SmallDFT<R1, SIGN>::run(t);
#pragma unroll
		for (int k1 = 0; k1 < R1; ++k1) {
			float2 x = t[k1];
			if (n2 * k1 != 0) {
				const float2 w = root<R>(n2 * k1);
				x = cmul(x, make_float2(w.x, static_cast<float>(SIGN) * w.y));
			}
			a[n2 * R1 + k1] = x;
		}
	}
#pragma unroll
	for (int k1 = 0; k1 < R1; ++k1) {
		float2 t[R2];
#pragma unroll
		for (int n2 = 0; n2 < R2; ++n2) t[n2] = a[n2 * R1 + k1];
		SmallDFT<R2, SIGN>::run(t);
#pragma unroll
		for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = t[k2];
	}
}
template<int SIGN> struct SmallDFT<6, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<3, 2, SIGN>(v); }
};
template<int SIGN> struct SmallDFT<9, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<3, 3, SIGN>(v); }
};
template<int SIGN> struct SmallDFT<15, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<5, 3, SIGN>(v); }
};
template<int SIGN> struct SmallDFT<16, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<4, 4, SIGN>(v); }
};
template<int SIGN> struct SmallDFT<10, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<5, 2, SIGN>(v); }
};
template<int SIGN> struct SmallDFT<12, SIGN> {
	static __device__ __forceinline__ void run(float2* v) { composite_dft<4, 3, SIGN>(v); }
};

// W^m from the two-level table in shared memory.
__device__ __forceinline__ float2 twiddle(const float2* lo, const float2* hi, unsigned m)
{
	return cmul(hi[m / kTwiddleSplit], lo[m % kTwiddleSplit]);
}

// w[q] = w[1]^q for q = 2 .. R-1, as w[q/2] w[q - q/2] (about log2(q)
// products deep).
template<int R>
__device__ __forceinline__ void twiddle_powers(float2* w)
{
#pragma unroll
	for (int q = 2; q < R; ++q) w[q] = cmul(w[q / 2], w[q - q / 2]);
}

// One component (c = 0: real, 1: imaginary) of complex output sample n,
// rounded as Complex<S>::pack rounds it.
template<int S>
__device__ __forceinline__ void store_component(typename Complex<S>::T* out, size_t n, int c, float v)
{
	if constexpr (S == STORE_F16) {
		reinterpret_cast<__half*>(out)[2 * n + c] = __float2half_rn(v);
	} else if constexpr (S == STORE_BF16) {
		reinterpret_cast<__nv_bfloat16*>(out)[2 * n + c] = __float2bfloat16_rn(v);
	} else {
		reinterpret_cast<float*>(out)[2 * n + c] = v;
	}
}

// One in-place stage over `data` (M points), blocks of span Ms, radix R.
// Forward (DIF): DFT_R of the R inputs at stride Ms/R, then twiddle
// W_Ms^(q j). Inverse (DIT, the transpose): conjugate twiddle, then DFT_R.
// W_Ms^j comes from the stage's own table `st` (consecutive j in consecutive
// lanes: no bank conflicts) or, without one, from the two-level table; its
// powers are formed in registers. The last stage (Ms = R) has no twiddles;
// elsewhere j = 0 multiplies by exactly 1.
template<int R, bool INVERSE>
__device__ __forceinline__ void fft_stage(float2* data, const float2* twLo, const float2* twHi, const float2* st,
		unsigned M, unsigned Ms, unsigned long long magic)
{
	const unsigned sub = Ms / R;
	const unsigned twStride = M / Ms;
	const unsigned nb = M / R;
	const bool twiddled = sub > 1;
	for (unsigned b = threadIdx.x; b < nb; b += blockDim.x) {
		const unsigned blk = static_cast<unsigned>((static_cast<unsigned long long>(b) * magic) >> 40);
		const unsigned j = b - blk * sub;
		const unsigned base = blk * Ms + j;
		float2 v[R];
#pragma unroll
		for (int q = 0; q < R; ++q) v[q] = data[base + q * sub];
		// The powers of W are formed next to their use (the forward stage
		// after its DFT), so that the R inputs and R powers are not all live
		// at once.
		float2 w[R];
		if (twiddled) w[1] = st ? st[j] : twiddle(twLo, twHi, j * twStride);
		if (!INVERSE) {
			SmallDFT<R, -1>::run(v);
			if (twiddled) {
				twiddle_powers<R>(w);
#pragma unroll
				for (int q = 1; q < R; ++q) v[q] = cmul(v[q], w[q]);
			}
		} else {
			if (twiddled) {
				twiddle_powers<R>(w);
#pragma unroll
				for (int q = 1; q < R; ++q) v[q] = cmulc(v[q], w[q]);
			}
			SmallDFT<R, +1>::run(v);
		}
#pragma unroll
		for (int q = 0; q < R; ++q) data[base + q * sub] = v[q];
	}
}

template<bool INVERSE>
__device__ __noinline__ void fft_run(float2* data, const PrepParams& p, const float2* twLo, const float2* twHi, const float2* stw)
{
	unsigned spans[kMaxFFTStages];
	unsigned Ms = p.M;
	for (int s = 0; s < p.numStages; ++s) { spans[s] = Ms; Ms /= p.radix[s]; }
	for (int i = 0; i < p.numStages; ++i) {
		const int s = INVERSE ? p.numStages - 1 - i : i;
		const float2* st = (stw && s > 0) ? stw + p.stwOffset[s] : nullptr;
		switch (p.radix[s]) {
		case 2: fft_stage<2, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 3: fft_stage<3, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 4: fft_stage<4, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 5: fft_stage<5, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 6: fft_stage<6, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 8: fft_stage<8, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 9: fft_stage<9, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 10: fft_stage<10, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 12: fft_stage<12, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		case 15: fft_stage<15, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		default: fft_stage<16, INVERSE>(data, twLo, twHi, st, p.M, spans[s], p.divMagic[s]); break;
		}
		__syncthreads();
	}
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

// Shared-memory layout of the prep kernels (float offsets).
struct PrepLayout {
	unsigned data, rfs, taps, twLo, twHi, stw, red, total;
	__host__ __device__ PrepLayout(const PrepParams& p, bool analytic)
	{
		const unsigned K = (p.tapsPerPhase - 1) / 2;
		data = 0;
		rfs = analytic ? ((2 * p.M + 3) & ~3u) : 0;   // 16-byte aligned for float4 taps after it
		taps = rfs + ((p.ns + 2 * K + 1 + 3) & ~3u);
		twLo = taps + p.U * p.tapsStride;
		twHi = twLo + (analytic ? 2 * kTwiddleSplit : 0);
		stw = twHi + (analytic ? 2 * p.twHiCount : 0);
		red = stw + ((analytic && p.stw) ? 2 * p.stwCount : 0);
		total = red + 32;
	}
};

// Loads the A-scan into shared memory with K zeros on each side (and one
// spare zero at the end), the polyphase taps and the twiddle tables.
// tables: also the taps and twiddle tables (false: they are still in shared
// memory from the previous A-scan of the same frame).
__device__ void load_inputs(const PrepParams& p, const PrepLayout& lay, float* sm, const float* __restrict__ rf,
		bool analytic, bool tables = true)
{
	const unsigned K = (p.tapsPerPhase - 1) / 2;
	float* rfs = sm + lay.rfs;
	const unsigned total = p.ns + 2 * K + 1;
	for (unsigned i = threadIdx.x; i < total; i += blockDim.x) {
		const int j = static_cast<int>(i) - static_cast<int>(K);
		rfs[i] = (j >= 0 && j < static_cast<int>(p.ns)) ? __ldg(&rf[j]) : 0.f;
	}
	float* taps = sm + lay.taps;
	if (!tables) {
		__syncthreads();
		return;
	}
	for (unsigned i = threadIdx.x; i < p.U * p.tapsStride; i += blockDim.x) taps[i] = __ldg(&p.polyTaps[i]);
	if (analytic) {
		const unsigned ntw = 2 * (kTwiddleSplit + p.twHiCount);
		const float* twg = reinterpret_cast<const float*>(p.tw);
		for (unsigned i = threadIdx.x; i < ntw; i += blockDim.x) sm[lay.twLo + i] = __ldg(&twg[i]);
		if (p.stw) {
			const float* stg = reinterpret_cast<const float*>(p.stw);
			for (unsigned i = threadIdx.x; i < 2 * p.stwCount; i += blockDim.x) sm[lay.stw + i] = __ldg(&stg[i]);
		}
	}
	__syncthreads();
}

// 16-byte shared-memory load the compiler may not hoist out of the sample
// loop (hoisting all U x 28 taps would exhaust the registers).
__device__ __forceinline__ float4 lds_taps(const float* p)
{
	float4 v;
	asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
			: "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(smem_addr(p)));
	return v;
}

// Four taps from shared memory, or (PT) from the launch parameters, where the
// compile-time offsets make them constant-bank operands of the FMAs.
template<bool PT>
__device__ __forceinline__ float4 tap4(const float* h)
{
	if constexpr (PT) {
		return make_float4(h[0], h[1], h[2], h[3]);
	} else {
		return lds_taps(h);
	}
}

// Whether a specialised FIR shape's taps fit in PrepParams::paramTaps.
template<int NT, int U>
__host__ __device__ constexpr bool param_taps_fit() { return NT > 0 && U * ((NT + 3) & ~3) <= static_cast<int>(kParamTaps); }

// The U upsampled outputs of input position b: x[bU + r] = sum_t h[r][t] *
// rf[b + K - t] (rfs holds rf shifted by K).
template<int NT, int U, bool PT = false>
__device__ __forceinline__ void fir_outputs(const float* rfs, const float* taps, unsigned b, float* out)
{
	constexpr int NTP = (NT + 3) & ~3;
	float win[NTP];
#pragma unroll
	for (int t = 0; t < NT; ++t) win[t] = rfs[b + (NT - 1) - t];
#pragma unroll
	for (int t = NT; t < NTP; ++t) win[t] = 0.f;
#pragma unroll
	for (int r = 0; r < U; ++r) {
		const float* h = taps + r * NTP;
		float acc = 0.f;
#pragma unroll
		for (int q = 0; q < NTP / 4; ++q) {
			const float4 c = tap4<PT>(h + 4 * q);
			acc = fmaf(c.x, win[4 * q], acc);
			if (4 * q + 1 < NT) acc = fmaf(c.y, win[4 * q + 1], acc);
			if (4 * q + 2 < NT) acc = fmaf(c.z, win[4 * q + 2], acc);
			if (4 * q + 3 < NT) acc = fmaf(c.w, win[4 * q + 3], acc);
		}
		out[r] = acc;
	}
}

// Generic form (any FIR length and factor).
__device__ __forceinline__ float fir_one(const float* rfs, const float* taps, unsigned n, unsigned U, unsigned nt,
		unsigned stride)
{
	const unsigned b = n / U;
	const unsigned r = n - b * U;
	const float* h = taps + r * stride;
	const float* src = rfs + b + (nt - 1);
	float acc = 0.f;
	for (unsigned t = 0; t < nt; ++t) acc = fmaf(h[t], src[-static_cast<int>(t)], acc);
	return acc;
}

// Pass 1: x[n] for n < L into xs (float view), partial sum of [deadZone, L).
// fir_outputs for two input positions b0 and b1 at once: each broadcast tap
// load serves both windows (half the tap traffic of two single calls).
template<int NT, int U, bool PT>
__device__ __forceinline__ void fir_outputs2(const float* rfs, const float* taps, unsigned b0, unsigned b1,
		float* out0, float* out1)
{
	constexpr int NTP = (NT + 3) & ~3;
	float w0[NTP], w1[NTP];
#pragma unroll
	for (int t = 0; t < NT; ++t) {
		w0[t] = rfs[b0 + (NT - 1) - t];
		w1[t] = rfs[b1 + (NT - 1) - t];
	}
#pragma unroll
	for (int t = NT; t < NTP; ++t) w0[t] = w1[t] = 0.f;
#pragma unroll
	for (int r = 0; r < U; ++r) {
		const float* h = taps + r * NTP;
		float a0 = 0.f, a1 = 0.f;
#pragma unroll
		for (int q = 0; q < NTP / 4; ++q) {
			const float4 c = tap4<PT>(h + 4 * q);
			a0 = fmaf(c.x, w0[4 * q], a0);
			a1 = fmaf(c.x, w1[4 * q], a1);
			if (4 * q + 1 < NT) { a0 = fmaf(c.y, w0[4 * q + 1], a0); a1 = fmaf(c.y, w1[4 * q + 1], a1); }
			if (4 * q + 2 < NT) { a0 = fmaf(c.z, w0[4 * q + 2], a0); a1 = fmaf(c.z, w1[4 * q + 2], a1); }
			if (4 * q + 3 < NT) { a0 = fmaf(c.w, w0[4 * q + 3], a0); a1 = fmaf(c.w, w1[4 * q + 3], a1); }
		}
		out0[r] = a0;
		out1[r] = a1;
	}
}

// The U outputs of input position b: into xs (the packed buffer read as
// floats) and the running DC sum of [deadZone, L).
template<int U>
__device__ __forceinline__ void fir_keep(const PrepParams& p, unsigned b, const float* o, float* xs, float& part)
{
#pragma unroll
	for (int r = 0; r < U; ++r) {
		if (b * U + r >= p.deadZone) part += o[r];
	}
	if (xs) {
		if constexpr (U % 4 == 0) {
#pragma unroll
			for (int r = 0; r < U; r += 4) {
				*reinterpret_cast<float4*>(xs + b * U + r) = make_float4(o[r], o[r + 1], o[r + 2], o[r + 3]);
			}
		} else {
#pragma unroll
			for (int r = 0; r < U; ++r) xs[b * U + r] = o[r];
		}
	}
}

template<int NT, int U, bool PT>
__device__ float fir_pass(const PrepParams& p, const float* rfs, const float* taps, float* xs)
{
	float part = 0.f;
	if constexpr (NT > 1) {
		// Input positions b and b + blockDim.x together.
		for (unsigned b = threadIdx.x; b < p.ns; b += 2 * blockDim.x) {
			const unsigned b1 = b + blockDim.x;
			const bool two = b1 < p.ns;
			float o0[U], o1[U];
			fir_outputs2<NT, U, PT>(rfs, taps, b, two ? b1 : b, o0, o1);
			fir_keep<U>(p, b, o0, xs, part);
			if (two) fir_keep<U>(p, b1, o1, xs, part);
		}
	} else if constexpr (NT > 0) {
		for (unsigned b = threadIdx.x; b < p.ns; b += blockDim.x) {
			float o[U];
			fir_outputs<NT, U, PT>(rfs, taps, b, o);
			fir_keep<U>(p, b, o, xs, part);
		}
	} else {
		for (unsigned n = threadIdx.x; n < p.L; n += blockDim.x) {
			const float x = fir_one(rfs, taps, n, p.U, p.tapsPerPhase, p.tapsStride);
			if (n >= p.deadZone) part += x;
			if (xs) xs[n] = x;
		}
	}
	return part;
}


// Imaginary parts y[n] / M of the analytic output (the real parts were
// written by the DC-removal pass).
template<int S>
__device__ void store_imag_pass(const PrepParams& p, const float* ys, unsigned a)
{
	using CT = typename Complex<S>::T;
	CT* out = reinterpret_cast<CT*>(p.out) + static_cast<size_t>(a) * p.outStride;
	const float invM = 1.0f / static_cast<float>(p.M);
	const float sc = p.outScale;
	for (unsigned n = threadIdx.x; n < p.L; n += blockDim.x) store_component<S>(out, n, 1, ys[n] * invM * sc);
}

// Store pass of the real-RF path: x[n] - mean, with x recomputed from the A-scan.
template<int S, int NT, int U, bool PT>
__device__ void store_real_pass(const PrepParams& p, const float* rfs, const float* taps, float mean, unsigned a)
{
	const float sc = p.outScale;
	using RT = typename Real<S>::T;
	RT* out = reinterpret_cast<RT*>(p.out) + static_cast<size_t>(a) * p.outStride;
	if constexpr (NT > 0) {
		for (unsigned b = threadIdx.x; b < p.ns; b += blockDim.x) {
			float o[U];
			fir_outputs<NT, U, PT>(rfs, taps, b, o);
#pragma unroll
			for (int r = 0; r < U; ++r) out[b * U + r] = Real<S>::pack((o[r] - mean) * sc);
		}
	} else {
		for (unsigned n = threadIdx.x; n < p.L; n += blockDim.x) {
			out[n] = Real<S>::pack((fir_one(rfs, taps, n, p.U, p.tapsPerPhase, p.tapsStride) - mean) * sc);
		}
	}
}

// The Hilbert multiplier of the pair whose table entry h sits at position i
// (PrepParams::hilb): W[k_lo] and W[M - k_lo] in place, or W[0] = 0, or
// W[M/2] = i Z[M/2].
constexpr int kHilbertBatch = 4;
__device__ __forceinline__ void hilbert_pair(float2* data, unsigned i, const float4& h)
{
	const unsigned code = __float_as_uint(h.z);
	if (code == kHilbertSkip) return;
	if (code == i) {
		if (i == 0) {
			data[0] = make_float2(0.f, 0.f);   // k = 0 sits at position 0
		} else {
			const float2 z = data[i];          // k = M / 2
			data[i] = make_float2(-z.y, z.x);
		}
		return;
	}
	const unsigned q = code & ~kHilbertSwap;
	const bool swap = (code & kHilbertSwap) != 0u;
	const unsigned q1 = swap ? q : i;      // position of k_lo
	const unsigned q2 = swap ? i : q;      // position of M - k_lo
	const float2 A = data[q1], B = data[q2];
	const float2 cs = make_float2(h.x, h.y);
	data[q1] = make_float2(cs.x * B.x - cs.y * A.y, cs.y * A.x - cs.x * B.y);
	data[q2] = make_float2(-cs.y * B.y - cs.x * A.x, cs.y * B.x + cs.x * A.y);
}

// y[n] - mean for the U outputs of input position b: into xs (analytic path,
// the FFT buffer; prep_analytic_tail stores them to the output) or into the
// real output.
template<int S, int U, bool ANALYTIC>
__device__ __forceinline__ void fir_store_dc_free(const PrepParams& p, unsigned b, const float* o, float mean,
		float* xs, void* outRow)
{
	const float sc = p.outScale;
	float d[U];
#pragma unroll
	for (int r = 0; r < U; ++r) d[r] = o[r] - mean;
	if constexpr (ANALYTIC) {
		if constexpr (U % 4 == 0) {
#pragma unroll
			for (int r = 0; r < U; r += 4) *reinterpret_cast<float4*>(xs + b * U + r) = make_float4(d[r], d[r + 1], d[r + 2], d[r + 3]);
		} else {
#pragma unroll
			for (int r = 0; r < U; ++r) xs[b * U + r] = d[r];
		}
	} else {
		using RT = typename Real<S>::T;
		RT* out = reinterpret_cast<RT*>(outRow) + static_cast<size_t>(b) * U;
		if constexpr (S == STORE_F32 && U % 4 == 0) {
#pragma unroll
			for (int r = 0; r < U; r += 4) {
				*reinterpret_cast<float4*>(out + r) = make_float4(d[r] * sc, d[r + 1] * sc, d[r + 2] * sc, d[r + 3] * sc);
			}
		} else {
#pragma unroll
			for (int r = 0; r < U; ++r) out[r] = Real<S>::pack(d[r] * sc);
		}
	}
}

// The real parts of the analytic output, (x[n] * scale, 0) for n < L, from the
// DC-free signal in xs, one sample a thread and step: consecutive threads
// store consecutive 8-byte samples (measured twice as fast per byte as
// 16-byte stores of two samples), every 32-byte sector written whole (the
// imaginary halves merge into the lines in L2 later).
template<int S>
__device__ void store_real_parts(const PrepParams& p, const float* xs, void* outRow)
{
	using CT = typename Complex<S>::T;
	CT* out = reinterpret_cast<CT*>(outRow);
	const float sc = p.outScale;
	for (unsigned n = threadIdx.x; n < p.L; n += blockDim.x) out[n] = Complex<S>::pack(xs[n] * sc, 0.0f);
}

// The mean of [deadZone, L) from the inputs: sum_i x[i] dc[i] / count, in
// an order that does not depend on the block size (128 partial sums over
// i = j mod 128, folded in a fixed tree), so that every kernel preparing an
// A-scan takes the same mean. Contains the block's barriers.
__device__ float dc_mean(const float* x, const float* dc, unsigned n, float* red, float count)
{
	float v = 0.f;
	if (threadIdx.x < 128) {
		for (unsigned i = threadIdx.x; i < n; i += 128) v = fmaf(x[i], dc[i], v);
	}
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	const unsigned warp = threadIdx.x >> 5;
	if ((threadIdx.x & 31) == 0 && warp < 4) red[warp] = v;
	__syncthreads();
	const float r = ((red[0] + red[1]) + (red[2] + red[3])) / count;
	__syncthreads();
	return r;
}

// FIR pass with the DC removed (the mean known beforehand): the DC-free
// signal into xs and, analytic path, (real, 0) into the output row; real
// path, the output row itself.
template<int S, int NT, int U, bool PT, bool ANALYTIC>
__device__ __forceinline__ void fir_dc_free_pass(const PrepParams& p, const float* rfs, const float* taps, float mean,
		float* xs, void* outRow)
{
	if constexpr (NT > 1) {
		for (unsigned b = threadIdx.x; b < p.ns; b += 2 * blockDim.x) {
			const unsigned b1 = b + blockDim.x;
			const bool two = b1 < p.ns;
			float o0[U], o1[U];
			fir_outputs2<NT, U, PT>(rfs, taps, b, two ? b1 : b, o0, o1);
			fir_store_dc_free<S, U, ANALYTIC>(p, b, o0, mean, xs, outRow);
			if (two) fir_store_dc_free<S, U, ANALYTIC>(p, b1, o1, mean, xs, outRow);
		}
	} else {
		for (unsigned b = threadIdx.x; b < p.ns; b += blockDim.x) {
			float o[U];
			fir_outputs<NT, U, PT>(rfs, taps, b, o);
			fir_store_dc_free<S, U, ANALYTIC>(p, b, o, mean, xs, outRow);
		}
	}
}

// Hilbert multiplier and real-FFT split, on the pairs (k, M-k):
// W[k] = i sin(pi k/M) Z[k] + cos(pi k/M) conj(Z[M-k]), W[0] = 0, visited in
// digit-reversed position order (both members of neighbouring lanes' pairs
// sit at neighbouring positions). A thread loads the table entries of
// kHilbertBatch pairs before it works on them, so their L2 latencies overlap
// (the pairs are disjoint).
__device__ __forceinline__ void hilbert_pass(const PrepParams& p, float2* data)
{
	for (unsigned i0 = threadIdx.x; i0 < p.hilbCount; i0 += kHilbertBatch * blockDim.x) {
		float4 h[kHilbertBatch];
#pragma unroll
		for (int u = 0; u < kHilbertBatch; ++u) {
			const unsigned i = i0 + u * blockDim.x;
			h[u] = (i < p.hilbCount) ? __ldg(&p.hilb[i]) : make_float4(0.f, 0.f, __uint_as_float(kHilbertSkip), 0.f);
		}
#pragma unroll
		for (int u = 0; u < kHilbertBatch; ++u) hilbert_pair(data, i0 + u * blockDim.x, h[u]);
	}
}

// Steps 3-6 of the analytic path after the DC-free signal is in the buffer:
// the real parts of the output row (x[n] * scale, 0) stored, forward FFT
// (digit-reversed output), Hilbert multiplier and real-FFT split, inverse
// FFT (natural-order output: y[n] * M at float index n), the imaginary parts
// y[n] / M * scale stored, and a barrier (shared memory is reused by the next
// A-scan). The stores take passes of their own: folded into the outermost
// FFT stages they share the load/store pipe with the butterflies' shared
// memory traffic and measured slower (cf2d: 30.4 k -> 41.5 k cycles forward,
// 29.5 k -> 39.0 k inverse, per A-scan).
template<int S>
__device__ void prep_analytic_tail(const PrepParams& p, unsigned a, float2* data, const float* xs, const float2* twLo,
		const float2* twHi, const float2* stw)
{
	store_real_parts<S>(p, xs, reinterpret_cast<typename Complex<S>::T*>(p.out) + static_cast<size_t>(a) * p.outStride);
	__syncthreads();
	fft_run<false>(data, p, twLo, twHi, stw);
	hilbert_pass(p, data);
	__syncthreads();
	fft_run<true>(data, p, twLo, twHi, stw);
	store_imag_pass<S>(p, xs, a);
	__syncthreads();
}

// Tensor-memory columns a thread needs for L samples, one per step of T
// threads (ceil(L / T) rounded up to 8), and a block's allocation: the
// T / 128 warps of an SM sub-partition side by side, as a power of two >= 32.
__host__ __device__ inline unsigned tmem_thread_columns(unsigned L, unsigned T)
{
	return ((L + T - 1) / T + 7) & ~7u;
}
__host__ __device__ inline unsigned tmem_block_columns(unsigned L, unsigned T)
{
	const unsigned need = tmem_thread_columns(L, T) * (T / 128);
	unsigned c = 32;
	while (c < need) c <<= 1;
	return c;
}

// prep_analytic_tail with the real parts parked in tensor memory: this
// thread's samples x[n], n = threadIdx.x + T j, go to its TMEM lane (columns
// tcol + j) before the FFTs overwrite the buffer, and one pass after the
// inverse FFT stores whole complex samples (x[n] * scale, y[n] / M * scale):
// the same values as the two store passes, in one. Those passes are bound by
// the SM's store path (about 8 cycles a warp store instruction, whatever its
// width), so the second pass's 4-byte stores cost as much as whole samples.
template<int S, int T>
__device__ void prep_analytic_tail_tmem(const PrepParams& p, unsigned a, float2* data, const float* xs,
		const float2* twLo, const float2* twHi, const float2* stw, uint32_t tcol)
{
	const unsigned L = p.L;
	const unsigned J8 = tmem_thread_columns(L, T);
	for (unsigned c = 0; c < J8; c += 8) {
		float v[8];
#pragma unroll
		for (int i = 0; i < 8; ++i) {
			const unsigned n = threadIdx.x + T * (c + i);
			v[i] = n < L ? xs[n] : 0.0f;
		}
		__syncwarp();
		tmem_store8(tcol + c, v);
	}
	__syncthreads();
	fft_run<false>(data, p, twLo, twHi, stw);
	hilbert_pass(p, data);
	__syncthreads();
	fft_run<true>(data, p, twLo, twHi, stw);
	using CT = typename Complex<S>::T;
	CT* out = reinterpret_cast<CT*>(p.out) + static_cast<size_t>(a) * p.outStride;
	const float invM = 1.0f / static_cast<float>(p.M);
	const float sc = p.outScale;
	for (unsigned c = 0; c < J8; c += 8) {
		float v[8];
		__syncwarp();
		tmem_load8(tcol + c, v);
#pragma unroll
		for (int i = 0; i < 8; ++i) {
			const unsigned n = threadIdx.x + T * (c + i);
			if (n < L) out[n] = Complex<S>::pack(v[i] * sc, xs[n] * invM * sc);
		}
	}
	__syncthreads();
}

// Analytic path, one A-scan `a` of the frame described by p. NT = 0 selects
// the generic FIR loop. ENV: the envelope of the input itself instead
// (HilbertEnvelope::calculate: no DC removal, |analytic signal| as floats;
// used with U = 1 on image columns). PT: FIR taps from p.paramTaps (p a
// launch parameter) instead of shared memory. PARK_T > 0 (a block of PARK_T
// threads holding tensor memory, `tlane` = its base address with this warp's
// lane field): with p.tmemCols set, the real parts wait in tensor memory
// (prep_analytic_tail_tmem).
template<int S, int NT, int U, bool ENV = false, bool PT = false, int PARK_T = 0>
__device__ void prep_analytic_body(const PrepParams& p, unsigned a, float* sm, bool tables = true, uint32_t tlane = 0)
{
	const PrepLayout lay(p, true);
	load_inputs(p, lay, sm, p.rf + static_cast<size_t>(a) * p.ns, true, tables);
	float2* data = reinterpret_cast<float2*>(sm + lay.data);
	float* xs = sm + lay.data;  // the packed complex buffer read as floats: x[n] at n
	const float* rfs = sm + lay.rfs;
	const float* taps = PT ? p.paramTaps : sm + lay.taps;
	const float2* twLo = reinterpret_cast<const float2*>(sm + lay.twLo);
	const float2* twHi = reinterpret_cast<const float2*>(sm + lay.twHi);
	const float2* stw = p.stw ? reinterpret_cast<const float2*>(sm + lay.stw) : nullptr;
	const unsigned L = p.L;

	// 1. Upsampled signal into the packed buffer, zero past L.
	for (unsigned n = L + threadIdx.x; n < 2 * p.M; n += blockDim.x) xs[n] = 0.f;
	if constexpr (!ENV && NT > 0) {
		if (p.dcCoef) {
			// The mean from the inputs (PrepParams::dcCoef), the DC removed
			// inside the FIR pass, as the single-frame stream kernel does.
			const unsigned K = (NT - 1) / 2;
			const float m = dc_mean(rfs + K, p.dcCoef, p.ns, sm + lay.red, static_cast<float>(L - p.deadZone));
			void* outRow = reinterpret_cast<typename Complex<S>::T*>(p.out) + static_cast<size_t>(a) * p.outStride;
			fir_dc_free_pass<S, NT, U, PT, true>(p, rfs, taps, m, xs, outRow);
			__syncthreads();
			if constexpr (PARK_T > 0) {
				if (p.tmemCols) {
					const uint32_t tcol = tlane + (threadIdx.x >> 7) * tmem_thread_columns(L, PARK_T);
					prep_analytic_tail_tmem<S, PARK_T>(p, a, data, xs, twLo, twHi, stw, tcol);
					return;
				}
			}
			prep_analytic_tail<S>(p, a, data, xs, twLo, twHi, stw);
			return;
		}
	}
	const float part = fir_pass<NT, U, PT>(p, rfs, taps, xs);
	// 2. DC removal: mean of [deadZone, L) subtracted from all L samples
	//    (block_sum's barriers also order the writes above). The real parts
	//    of the output, (x[n] - mean) * scale, are stored with the first FFT
	//    stage (prep_analytic_tail) as whole complex samples with a zero
	//    imaginary part, so that every 32-byte sector is written whole: a
	//    sector holding only real halves was written back to HBM partially
	//    and read back when the imaginary parts arrived, 0.7 GB each way per
	//    cf2d frame. The imaginary parts then merge into the lines in L2.
	float mean = 0.f;
	if constexpr (!ENV) {
		mean = block_sum(part, sm + lay.red) / static_cast<float>(L - p.deadZone);
		for (unsigned n = threadIdx.x; n < L; n += blockDim.x) xs[n] -= mean;
	}
	__syncthreads();

	if constexpr (!ENV) {
		prep_analytic_tail<S>(p, a, data, xs, twLo, twHi, stw);
		return;
	}
	// 3. Forward FFT (digit-reversed output).
	fft_run<false>(data, p, twLo, twHi, stw);
	// 4. Hilbert multiplier and real-FFT split (hilbert_pass).
	hilbert_pass(p, data);
	__syncthreads();
	// 5. Inverse FFT (natural-order output: y[n] * M at float index n).
	fft_run<true>(data, p, twLo, twHi, stw);
	// 6. |x[n] + i y[n]|.
	{
		// |x[n] + i y[n]| (the input itself is the real part).
		const float invM = 1.0f / static_cast<float>(p.M);
		float* out = reinterpret_cast<float*>(p.out) + static_cast<size_t>(a) * p.outStride;
		for (unsigned n = threadIdx.x; n < L; n += blockDim.x) {
			const float x = rfs[n];
			const float y = xs[n] * invM;
			out[n] = sqrtf(x * x + y * y);
		}
	}
	__syncthreads();  // shared memory is reused by the next A-scan of a batch
}

// Real-RF path: upsampling (fixed 4x FIR) and DC removal only.
template<int S, int NT, int U, bool PT = false>
__device__ void prep_real_body(const PrepParams& p, unsigned a, float* sm, bool tables = true)
{
	const PrepLayout lay(p, false);
	load_inputs(p, lay, sm, p.rf + static_cast<size_t>(a) * p.ns, false, tables);
	const float* taps = PT ? p.paramTaps : sm + lay.taps;
	if constexpr (NT > 0) {
		if (p.dcCoef) {
			const unsigned K = (NT - 1) / 2;
			const float m = dc_mean(sm + lay.rfs + K, p.dcCoef, p.ns, sm + lay.red, static_cast<float>(p.L - p.deadZone));
			fir_dc_free_pass<S, NT, U, PT, false>(p, sm + lay.rfs, taps, m, nullptr,
					reinterpret_cast<typename Real<S>::T*>(p.out) + static_cast<size_t>(a) * p.outStride);
			__syncthreads();
			return;
		}
	}
	const float part = fir_pass<NT, U, PT>(p, sm + lay.rfs, taps, nullptr);
	const float mean = block_sum(part, sm + lay.red) / static_cast<float>(p.L - p.deadZone);
	store_real_pass<S, NT, U, PT>(p, sm + lay.rfs, taps, mean, a);
	__syncthreads();
}

// Blocks of T threads, 512 / T of them per SM at most 128 registers a thread
// (short A-scans: several small blocks share an SM instead of one block of
// 512 threads with most of them idle in the FFT stages).
template<int S, int NT, int U, int T>
__global__ void __launch_bounds__(T, kPrepThreads / T)
prep_analytic_kernel(const __grid_constant__ PrepParams p)
{
	extern __shared__ __align__(16) float sm[];
	prep_analytic_body<S, NT, U, false, param_taps_fit<NT, U>()>(p, blockIdx.x, sm);
}

template<int S, int NT, int U, int T>
__global__ void __launch_bounds__(T, kPrepThreads / T)
prep_real_kernel(const __grid_constant__ PrepParams p)
{
	extern __shared__ __align__(16) float sm[];
	// (U = 8 on the real path would hold its 224 loop-invariant taps in
	// registers; that shape keeps them in shared memory.)
	prep_real_body<S, NT, U, param_taps_fit<NT, U>() && U <= 4>(p, blockIdx.x, sm);
}

// FIR shapes with specialised code: the processors' Kaiser-sinc FIR (half
// transition 0.2) has 2K + 1 = 27 taps per phase for every factor; the fixed
// 4x FIR of the real path has 21; no upsampling is 1 tap; 0 = generic.
__host__ __device__ inline int fir_shape(unsigned tapsPerPhase, unsigned U)
{
	if (tapsPerPhase == 27 && U == 8) return 1;
	if (tapsPerPhase == 27 && U == 4) return 2;
	if (tapsPerPhase == 21 && U == 4) return 3;
	if (tapsPerPhase == 1 && U == 1) return 4;
	return 0;
}

// ------------------------------------------------------------------ stream
// Single-frame launches of the specialised FIR shapes: persistent blocks
// (as many as the SMs hold) walk the frame's A-scans. Per block, once: the
// FIR taps, twiddle tables and DC weights into shared memory, and the zero
// margins of two input buffers. Per A-scan: its RF row arrives by bulk copy
// into one buffer while the previous A-scan is processed from the other
// (plain loads when the RF is not bulk-copyable, e.g. host memory read
// through the host's page tables); the DC mean of [deadZone, L) is the dot
// product of the row with PrepParams::dcCoef, so the FIR pass writes the
// DC-free signal in one pass: into the FFT buffer (analytic path; the tail
// stores its real parts, then transforms it) or as the output (real path).
struct StreamLayout {   // float offsets
	unsigned data, rfs[2], taps, twLo, twHi, stw, dc, red, bar, total;
	__host__ __device__ StreamLayout(const PrepParams& p, bool analytic)
	{
		const unsigned K = (p.tapsPerPhase - 1) / 2;
		data = 0;
		unsigned o = analytic ? ((2 * p.M + 3) & ~3u) : 0;
		// rfs[b][i] = rf[i - K]: K zeros, the row, K + 1 zeros; rfs + K is
		// 16-byte aligned (the bulk copy's destination).
		const unsigned pad = (4 - K % 4) % 4;
		const unsigned slot = (pad + 2 * K + p.ns + 1 + 3) & ~3u;
		rfs[0] = o + pad;
		rfs[1] = o + slot + pad;
		o += 2 * slot;
		taps = o;
		o += p.U * p.tapsStride;
		twLo = o;
		twHi = twLo + (analytic ? 2 * kTwiddleSplit : 0);
		stw = twHi + (analytic ? 2 * p.twHiCount : 0);
		dc = stw + ((analytic && p.stw) ? 2 * p.stwCount : 0);
		red = (dc + p.ns + 3) & ~3u;
		bar = red + 32;            // two mbarriers (16-byte aligned)
		total = bar + 4;
	}
};

constexpr unsigned long long kPrepWaitLimitNs = 2000000000ull;   // 2 s

template<int S, int NT, int U, int T, bool ANALYTIC>
__global__ void __launch_bounds__(T, kPrepThreads / T)
prep_stream_kernel(const __grid_constant__ PrepParams p)
{
	extern __shared__ __align__(16) float sm[];
	__shared__ int sAbort;
	__shared__ uint32_t sTmem;
	constexpr bool PT = param_taps_fit<NT, U>() && (ANALYTIC || U <= 4);
	// Only the 512-thread form (one block an SM) carries tensor-memory code.
	// The forms that share an SM measured slower with it: 128 threads (four
	// blocks an SM) 1.4-2.3x even where the launch left the parked path
	// unused, 256 threads (two blocks) 1.35x.
	constexpr bool kTmem = ANALYTIC && T == 512;
	const bool useTmem = kTmem && p.tmemCols != 0;
	constexpr unsigned K = (NT - 1) / 2;
	const StreamLayout lay(p, ANALYTIC);
	const unsigned ns = p.ns;
	uint64_t* bar = reinterpret_cast<uint64_t*>(sm + lay.bar);
	float* dc = sm + lay.dc;

	// Once per block: tables, DC weights, zero margins, barriers.
	for (unsigned i = threadIdx.x; i < p.U * p.tapsStride; i += T) sm[lay.taps + i] = __ldg(&p.polyTaps[i]);
	if constexpr (ANALYTIC) {
		const unsigned ntw = 2 * (kTwiddleSplit + p.twHiCount);
		const float* twg = reinterpret_cast<const float*>(p.tw);
		for (unsigned i = threadIdx.x; i < ntw; i += T) sm[lay.twLo + i] = __ldg(&twg[i]);
		if (p.stw) {
			const float* stg = reinterpret_cast<const float*>(p.stw);
			for (unsigned i = threadIdx.x; i < 2 * p.stwCount; i += T) sm[lay.stw + i] = __ldg(&stg[i]);
		}
	}
	for (unsigned i = threadIdx.x; i < ns; i += T) dc[i] = __ldg(&p.dcCoef[i]);
	for (int b = 0; b < 2; ++b) {
		float* rfs = sm + lay.rfs[b];
		for (unsigned i = threadIdx.x; i < 2 * K + 1; i += T) rfs[static_cast<int>(i) < static_cast<int>(K) ? i : ns + i] = 0.f;   // [0, K), [K + ns, 2K + ns + 1)
	}
	if (threadIdx.x == 0) {
		sAbort = 0;
		mbar_init(&bar[0], 1);
		mbar_init(&bar[1], 1);
		fence_barrier_init();
	}
	uint32_t tcol = 0;
	if constexpr (kTmem) {
		__syncwarp();
		if (useTmem && threadIdx.x < 32) tmem_alloc(&sTmem, p.tmemCols);
		tmem_fence_before_sync();
		__syncthreads();
		tmem_fence_after_sync();
		if (useTmem) {
			const unsigned w = threadIdx.x >> 5;
			tcol = sTmem + (((w & 3u) * 32u) << 16) + (w >> 2) * tmem_thread_columns(p.L, T);
		}
	} else {
		__syncthreads();
	}

	const bool bulk = p.rfBulk != 0;
	const unsigned rowBytes = ns * static_cast<unsigned>(sizeof(float));
	unsigned a = blockIdx.x;
	if (bulk && threadIdx.x == 0 && a < p.numSignals) {
		mbar_arrive_expect_tx(&bar[0], rowBytes);
		bulk_copy_g2s(sm + lay.rfs[0] + K, p.rf + static_cast<size_t>(a) * ns, rowBytes, &bar[0]);
	}
	const float* taps = PT ? p.paramTaps : sm + lay.taps;
	for (unsigned k = 0; a < p.numSignals; a += gridDim.x, ++k) {
		const unsigned cur = k & 1u;
		float* rfs = sm + lay.rfs[cur];
		if (bulk) {
			if (threadIdx.x == 0) {
				if (!mbar_wait_bounded(&bar[cur], (k >> 1) & 1u, kPrepWaitLimitNs)) {
					sAbort = 1;
					if (p.errWord) atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
				} else {
					// The next row into the other buffer (its last readers, the
					// previous A-scan's FIR pass, are past several barriers).
					const unsigned an = a + gridDim.x;
					if (an < p.numSignals) {
						fence_proxy_async_smem();
						mbar_arrive_expect_tx(&bar[cur ^ 1u], rowBytes);
						bulk_copy_g2s(sm + lay.rfs[cur ^ 1u] + K, p.rf + static_cast<size_t>(an) * ns, rowBytes,
								&bar[cur ^ 1u]);
					}
				}
			}
		} else {
			const float* row = p.rf + static_cast<size_t>(a) * ns;
			for (unsigned i = threadIdx.x; i < ns; i += T) rfs[K + i] = row[i];
		}
		__syncthreads();
		if (sAbort) break;   // the row never arrived; no copy is left in flight

		const float mean = dc_mean(rfs + K, dc, ns, sm + lay.red, static_cast<float>(p.L - p.deadZone));

		float* xs = sm + lay.data;
		void* outRow;
		if constexpr (ANALYTIC) {
			outRow = reinterpret_cast<typename Complex<S>::T*>(p.out) + static_cast<size_t>(a) * p.outStride;
			for (unsigned n = p.L + threadIdx.x; n < 2 * p.M; n += T) xs[n] = 0.f;
		} else {
			outRow = reinterpret_cast<typename Real<S>::T*>(p.out) + static_cast<size_t>(a) * p.outStride;
		}
		fir_dc_free_pass<S, NT, U, PT, ANALYTIC>(p, rfs, taps, mean, xs, outRow);
		__syncthreads();
		if constexpr (ANALYTIC) {
			float2* data = reinterpret_cast<float2*>(sm + lay.data);
			const float2* twLo = reinterpret_cast<const float2*>(sm + lay.twLo);
			const float2* twHi = reinterpret_cast<const float2*>(sm + lay.twHi);
			const float2* stw = p.stw ? reinterpret_cast<const float2*>(sm + lay.stw) : nullptr;
			if constexpr (kTmem) {
				if (useTmem) {
					prep_analytic_tail_tmem<S, T>(p, a, data, xs, twLo, twHi, stw, tcol);
					continue;
				}
			}
			prep_analytic_tail<S>(p, a, data, xs, twLo, twHi, stw);
		}
	}
	if constexpr (kTmem) {
		if (useTmem) {
			// Every thread's loads completed inside tmem_load8; the block's
			// columns go back before it exits.
			tmem_fence_before_sync();
			__syncthreads();
			tmem_fence_after_sync();
			__syncwarp();
			if (threadIdx.x < 32) tmem_dealloc(sTmem, p.tmemCols);
		}
	}
}

template<int S, int NT, int U, int T>
cudaError_t launch_stream_t(const PrepParams& p, bool analytic, size_t smem, cudaStream_t stream)
{
	const auto kernel = analytic ? prep_stream_kernel<S, NT, U, T, true> : prep_stream_kernel<S, NT, U, T, false>;
	cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
	if (e != cudaSuccess) return e;
	int perSM = 0, dev = 0, sms = 0;
	if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, T, smem)) != cudaSuccess) return e;
	if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
	if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
	const unsigned blocks = std::min(p.numSignals, static_cast<unsigned>(sms) * static_cast<unsigned>(perSM > 0 ? perSM : 1));
	// Tensor memory for the real parts (blocks of 512 threads, one an SM)
	// when the columns fit (an allocation never waits on this launch's own
	// blocks). Measured: cf2d (32768 samples an A-scan) 1.035 -> 0.970 ms,
	// 16384-sample A-scans 5-6 % faster.
	PrepParams q = p;
	q.tmemCols = 0;
	if (analytic && T == 512 && perSM <= 1) {
		const unsigned cols = tmem_block_columns(p.L, T);
		if (cols <= 512u && static_cast<unsigned>(perSM > 0 ? perSM : 1) * cols <= 512u) q.tmemCols = cols;
	}
	kernel<<<blocks, T, smem, stream>>>(q);
	return cudaGetLastError();
}

template<int S, int NT, int U>
cudaError_t launch_stream(const PrepParams& p, bool analytic, cudaStream_t stream)
{
	const size_t smem = static_cast<size_t>(StreamLayout(p, analytic).total) * sizeof(float);
	switch (prep_threads(smem)) {
	case 128: return launch_stream_t<S, NT, U, 128>(p, analytic, smem, stream);
	case 256: return launch_stream_t<S, NT, U, 256>(p, analytic, smem, stream);
	default: return launch_stream_t<S, NT, U, 512>(p, analytic, smem, stream);
	}
}

// Many frames: persistent blocks walk the A-scans of every frame of the batch.
template<int S, bool ANALYTIC, int T>
__global__ void __launch_bounds__(T, kPrepThreads / T)
prep_batch_kernel(const BatchPrepFrame* __restrict__ frames, const BatchHeader* __restrict__ hdr)
{
	extern __shared__ __align__(16) float sm[];
	__shared__ PrepParams sp;
	__shared__ uint32_t sTmem;
	static_assert(sizeof(PrepParams) % 8 == 0 && alignof(PrepParams) == 8, "PrepParams is copied as 8-byte words");
	const unsigned count = hdr->count;
	const unsigned total = hdr->totalSignals;
	unsigned f = 0, loaded = ~0u;
	// The 512-thread form (one block an SM) parks the real parts in tensor
	// memory when the launch asks for it (every frame's tmemCols: the columns
	// of the batch's longest A-scan); the forms that share an SM carry no
	// tensor-memory code (measured slower with it).
	constexpr bool kTmem = ANALYTIC && T == 512;
	constexpr int kParkT = kTmem ? T : 0;
	unsigned tmemCols = 0;
	uint32_t tlane = 0;
	if constexpr (kTmem) {
		tmemCols = count ? frames[0].prep.tmemCols : 0u;
		if (tmemCols && threadIdx.x < 32) tmem_alloc(&sTmem, tmemCols);
		tmem_fence_before_sync();
		__syncthreads();
		tmem_fence_after_sync();
		if (tmemCols) tlane = sTmem + ((((threadIdx.x >> 5) & 3u) * 32u) << 16);
	}
	for (unsigned g = blockIdx.x; g < total; g += gridDim.x) {
		while (f + 1 < count && frames[f + 1].signalBegin <= g) ++f;
		__syncthreads();  // the previous A-scan is done with sp
		// The frame's parameters into shared memory, by the whole block, and
		// its tables with its first A-scan here (consecutive A-scans of a
		// block mostly belong to one frame: only their RF rows are loaded).
		const bool tables = f != loaded;
		if (tables) {
			const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&frames[f].prep);
			unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sp);
			for (unsigned i = threadIdx.x; i < sizeof(PrepParams) / 8; i += blockDim.x) dst[i] = src[i];
			loaded = f;
		}
		__syncthreads();
		const unsigned a = g - frames[f].signalBegin;
		const int shape = fir_shape(sp.tapsPerPhase, sp.U);
		if (ANALYTIC) {
			switch (shape) {
			case 1: prep_analytic_body<S, 27, 8, false, false, kParkT>(sp, a, sm, tables, tlane); break;
			case 2: prep_analytic_body<S, 27, 4, false, false, kParkT>(sp, a, sm, tables, tlane); break;
			case 4: prep_analytic_body<S, 1, 1>(sp, a, sm, tables); break;
			default: prep_analytic_body<S, 0, 1>(sp, a, sm, tables); break;
			}
		} else {
			if (shape == 3) prep_real_body<S, 21, 4>(sp, a, sm, tables);
			else prep_real_body<S, 0, 1>(sp, a, sm, tables);
		}
	}
	if constexpr (kTmem) {
		if (tmemCols) {
			tmem_fence_before_sync();
			__syncthreads();
			tmem_fence_after_sync();
			__syncwarp();
			if (threadIdx.x < 32) tmem_dealloc(sTmem, tmemCols);
		}
	}
}

template<int S, int NT, int U, int T>
cudaError_t launch_kernel_t(const PrepParams& p, bool analytic, size_t smem, cudaStream_t stream)
{
	const dim3 grid(p.numSignals), block(T);
	cudaError_t e;
	if (analytic) {
		e = cudaFuncSetAttribute(prep_analytic_kernel<S, NT, U, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		prep_analytic_kernel<S, NT, U, T><<<grid, block, smem, stream>>>(p);
	} else {
		e = cudaFuncSetAttribute(prep_real_kernel<S, NT, U, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		prep_real_kernel<S, NT, U, T><<<grid, block, smem, stream>>>(p);
	}
	return cudaGetLastError();
}

template<int S, int NT, int U>
cudaError_t launch_kernel(const PrepParams& p, bool analytic, size_t smem, cudaStream_t stream)
{
	switch (prep_threads(smem)) {
	case 128: return launch_kernel_t<S, NT, U, 128>(p, analytic, smem, stream);
	case 256: return launch_kernel_t<S, NT, U, 256>(p, analytic, smem, stream);
	default: return launch_kernel_t<S, NT, U, 512>(p, analytic, smem, stream);
	}
}

template<int S>
cudaError_t dispatch_fir(const PrepParams& p, bool analytic, size_t smem, cudaStream_t stream)
{
	switch (fir_shape(p.tapsPerPhase, p.U)) {
	case 1: return launch_kernel<S, 27, 8>(p, analytic, smem, stream);
	case 2: return launch_kernel<S, 27, 4>(p, analytic, smem, stream);
	case 3: return launch_kernel<S, 21, 4>(p, analytic, smem, stream);
	case 4: return launch_kernel<S, 1, 1>(p, analytic, smem, stream);
	default: return launch_kernel<S, 0, 1>(p, analytic, smem, stream);
	}
}

template<int S, bool ANALYTIC, int T>
cudaError_t launch_batch_t(const BatchPrepFrame* frames, const BatchHeader* hdr, size_t smem, unsigned blocks,
		cudaStream_t stream)
{
	cudaError_t e = cudaFuncSetAttribute(prep_batch_kernel<S, ANALYTIC, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			static_cast<int>(smem));
	if (e != cudaSuccess) return e;
	prep_batch_kernel<S, ANALYTIC, T><<<blocks, T, smem, stream>>>(frames, hdr);
	return cudaGetLastError();
}

template<int S, bool ANALYTIC>
cudaError_t launch_batch(const BatchPrepFrame* frames, const BatchHeader* hdr, size_t smem, unsigned blocks,
		cudaStream_t stream)
{
	switch (prep_threads(smem)) {
	case 128: return launch_batch_t<S, ANALYTIC, 128>(frames, hdr, smem, blocks, stream);
	case 256: return launch_batch_t<S, ANALYTIC, 256>(frames, hdr, smem, blocks, stream);
	default: return launch_batch_t<S, ANALYTIC, 512>(frames, hdr, smem, blocks, stream);
	}
}

}  // namespace

size_t prep_smem_bytes(const PrepParams& p, bool analytic)
{
	return static_cast<size_t>(PrepLayout(p, analytic).total) * sizeof(float);
}

cudaError_t launch_prep_batch(const BatchPrepFrame* frames, const BatchHeader* hdr, size_t smem, unsigned blocks,
		int storage, bool analytic, cudaStream_t stream)
{
	if (analytic) {
		switch (storage) {
		case STORE_F16: return launch_batch<STORE_F16, true>(frames, hdr, smem, blocks, stream);
		case STORE_BF16: return launch_batch<STORE_BF16, true>(frames, hdr, smem, blocks, stream);
		default: return launch_batch<STORE_F32, true>(frames, hdr, smem, blocks, stream);
		}
	}
	switch (storage) {
	case STORE_F16: return launch_batch<STORE_F16, false>(frames, hdr, smem, blocks, stream);
	case STORE_BF16: return launch_batch<STORE_BF16, false>(frames, hdr, smem, blocks, stream);
	default: return launch_batch<STORE_F32, false>(frames, hdr, smem, blocks, stream);
	}
}

unsigned prep_batch_tmem_columns(size_t smem, unsigned maxL, bool analytic)
{
	if (!analytic || prep_threads(smem) != 512) return 0;
	const unsigned cols = tmem_block_columns(maxL, 512);
	return cols <= 512u ? cols : 0u;
}

int prep_threads(size_t smem)
{
	// Shared memory of an SM (228 KiB, 1 KiB reserved per block) over the block's.
	const size_t perSM = (228u * 1024u) / (smem + 1024u);
	return perSM >= 4 ? 128 : (perSM >= 2 ? 256 : 512);
}

// Envelope of numSignals real columns of ns samples (U = 1, single tap).
template<int T>
__global__ void __launch_bounds__(T, kPrepThreads / T)
envelope_kernel(PrepParams p)
{
	extern __shared__ __align__(16) float sm[];
	prep_analytic_body<STORE_F32, 1, 1, true>(p, blockIdx.x, sm);
}

template<int T>
cudaError_t launch_envelope_t(const PrepParams& p, size_t smem, cudaStream_t stream)
{
	cudaError_t e = cudaFuncSetAttribute(envelope_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
	if (e != cudaSuccess) return e;
	envelope_kernel<T><<<p.numSignals, T, smem, stream>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_envelope(const PrepParams& p, cudaStream_t stream)
{
	const size_t smem = prep_smem_bytes(p, true);
	switch (prep_threads(smem)) {
	case 128: return launch_envelope_t<128>(p, smem, stream);
	case 256: return launch_envelope_t<256>(p, smem, stream);
	default: return launch_envelope_t<512>(p, smem, stream);
	}
}

template<int S>
cudaError_t dispatch_stream(const PrepParams& p, bool analytic, cudaStream_t stream)
{
	switch (fir_shape(p.tapsPerPhase, p.U)) {
	case 1: return launch_stream<S, 27, 8>(p, analytic, stream);
	case 2: return launch_stream<S, 27, 4>(p, analytic, stream);
	case 3: return launch_stream<S, 21, 4>(p, analytic, stream);
	default: return launch_stream<S, 1, 1>(p, analytic, stream);
	}
}

bool prep_uses_stream(const PrepParams& p)
{
	return p.dcCoef != nullptr && fir_shape(p.tapsPerPhase, p.U) != 0;
}

size_t prep_stream_smem_bytes(const PrepParams& p, bool analytic)
{
	return static_cast<size_t>(StreamLayout(p, analytic).total) * sizeof(float);
}

cudaError_t launch_prep(const PrepParams& p, int storage, bool analytic, cudaStream_t stream)
{
	if (prep_uses_stream(p)) {
		switch (storage) {
		case STORE_F16: return dispatch_stream<STORE_F16>(p, analytic, stream);
		case STORE_BF16: return dispatch_stream<STORE_BF16>(p, analytic, stream);
		default: return dispatch_stream<STORE_F32>(p, analytic, stream);
		}
	}
	const size_t smem = prep_smem_bytes(p, analytic);
	switch (storage) {
	case STORE_F16: return dispatch_fir<STORE_F16>(p, analytic, smem, stream);
	case STORE_BF16: return dispatch_fir<STORE_BF16>(p, analytic, smem, stream);
	default: return dispatch_fir<STORE_F32>(p, analytic, smem, stream);
	}
}

}  // namespace usgb
