// Per-grid-point coherence-factor state over the terms (per-receiver sums of
// the STA kernels, single terms of the T1R1 / TnRn kernel), shared by the
// delay-and-sum kernels. P is any parameter block with pcfFactor and scfP.
#pragma once

#include "usgb_common.cuh"
#include "usgb_internal.h"

namespace usgb {

// Apodized sum of one receiver. The reference multiplies every gathered term
// by the weight (src/user/processor/VectorialSTAProcessor.h:279-281), so a
// receiver without any valid gather keeps +0 even when its weight is a tiny
// negative number (Blackman ends); + 0.0f turns the -0 of acc * weight into +0,
// which keeps atan2 (PCF) and the sign (SCF) of empty sums equal to the
// reference's.
__device__ __forceinline__ float2 receiver_sum(float2 acc, float w)
{
	return make_float2(fmaf(acc.x, w, 0.0f), fmaf(acc.y, w, 0.0f));
}

// |total| with explicit rounding (no contraction choice left to the
// compiler), so every kernel variant returns the same bits.
__device__ __forceinline__ float magnitude(float2 v)
{
	return __fsqrt_rn(__fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)));
}

template<int CF> struct CFState {
	__device__ void add(float2) {}
	template<class P> __device__ float result(unsigned, const P&, float2) const { return 1.0f; }
};

// PCF (src/util/CoherenceFactor.h:267-286): population standard deviation of
// the phases phi and of phi -+ pi, accumulated with Welford's update.
template<> struct CFState<CF_PCF> {
	unsigned n = 0;
	float m1 = 0.f, s1 = 0.f, m2 = 0.f, s2 = 0.f;
	__device__ void add(float2 v)
	{
		const float phi = atan2f(v.y, v.x);
		const float pi = 3.14159265358979323846f;
		const float aux = phi + ((phi < 0.f) ? pi : -pi);
		++n;
		const float inv = __frcp_rn(static_cast<float>(n));
		float d = __fsub_rn(phi, m1);
		m1 = __fmaf_rn(d, inv, m1);
		s1 = __fmaf_rn(d, __fsub_rn(phi, m1), s1);
		d = __fsub_rn(aux, m2);
		m2 = __fmaf_rn(d, inv, m2);
		s2 = __fmaf_rn(d, __fsub_rn(aux, m2), s2);
	}
	template<class P> __device__ float result(unsigned N, const P& p, float2) const
	{
		const float sd1 = __fsqrt_rn(__fdiv_rn(s1, static_cast<float>(N)));
		const float sd2 = __fsqrt_rn(__fdiv_rn(s2, static_cast<float>(N)));
		return fmaxf(0.f, __fsub_rn(1.f, __fmul_rn(p.pcfFactor, fminf(sd1, sd2))));
	}
};

// SCF (src/util/CoherenceFactor.h:217-236) on the real parts, sign(0) = +1.
template<> struct CFState<CF_SCF> {
	int signSum = 0;
	__device__ void add(float2 v) { signSum += (v.x >= 0.f) ? 1 : -1; }
	template<class P> __device__ float result(unsigned N, const P& p, float2) const
	{
		const float k = __fdiv_rn(static_cast<float>(signSum), static_cast<float>(N));
		const float m = __fsub_rn(1.f, __fsqrt_rn(__fsub_rn(1.f, __fmul_rn(k, k))));
		return powf(fabsf(m), p.scfP);
	}
};

// Mallart-Fink CF: |sum s|^2 / (N sum |s|^2) (not in the reference).
template<> struct CFState<CF_MF> {
	float energy = 0.f;
	__device__ void add(float2 v) { energy = __fmaf_rn(v.x, v.x, __fmaf_rn(v.y, v.y, energy)); }
	template<class P> __device__ float result(unsigned N, const P&, float2 total) const
	{
		if (energy == 0.f) return 0.f;
		const float num = __fadd_rn(__fmul_rn(total.x, total.x), __fmul_rn(total.y, total.y));
		return __fdiv_rn(num, __fmul_rn(static_cast<float>(N), energy));
	}
};

}  // namespace usgb
