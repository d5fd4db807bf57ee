// Per-grid-point coherence-factor state over the receivers, shared by the
// delay-and-sum kernels.
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

template<int CF> struct CFState {
	__device__ void add(float2) {}
	__device__ float result(unsigned, const DasParams&, float2) const { return 1.0f; }
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
		const float inv = 1.0f / static_cast<float>(n);
		float d = phi - m1;
		m1 += d * inv;
		s1 += d * (phi - m1);
		d = aux - m2;
		m2 += d * inv;
		s2 += d * (aux - m2);
	}
	__device__ float result(unsigned N, const DasParams& p, float2) const
	{
		const float sd1 = sqrtf(s1 / static_cast<float>(N));
		const float sd2 = sqrtf(s2 / static_cast<float>(N));
		return fmaxf(0.f, 1.f - p.pcfFactor * fminf(sd1, sd2));
	}
};

// SCF (src/util/CoherenceFactor.h:217-236) on the real parts, sign(0) = +1.
template<> struct CFState<CF_SCF> {
	int signSum = 0;
	__device__ void add(float2 v) { signSum += (v.x >= 0.f) ? 1 : -1; }
	__device__ float result(unsigned N, const DasParams& p, float2) const
	{
		const float k = static_cast<float>(signSum) / static_cast<float>(N);
		const float m = 1.f - sqrtf(1.f - k * k);
		return powf(fabsf(m), p.scfP);
	}
};

// Mallart-Fink CF: |sum s|^2 / (N sum |s|^2) (not in the reference).
template<> struct CFState<CF_MF> {
	float energy = 0.f;
	__device__ void add(float2 v) { energy = fmaf(v.x, v.x, fmaf(v.y, v.y, energy)); }
	__device__ float result(unsigned N, const DasParams&, float2 total) const
	{
		if (energy == 0.f) return 0.f;
		return (total.x * total.x + total.y * total.y) / (static_cast<float>(N) * energy);
	}
};

}  // namespace usgb
