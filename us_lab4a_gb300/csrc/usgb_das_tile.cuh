// Device helpers shared by the tiled delay-and-sum kernels (usgb_das_staged.cu,
// usgb_das_group.cu): sample codecs of the staged taps, the delay split into
// index and fraction (FP32 as the reference, or FP64 geometry in fixed
// point), and the gathers from a staged window or from global memory.
#pragma once

#include <cstdint>

#include "usgb_common.cuh"
#include "usgb_internal.h"

namespace usgb {
namespace tile {

constexpr int kGlobalWindow = -1;   // window too large for a stage: gather from global memory
constexpr int kEmptyWindow = -2;    // no valid sample can be reached
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

// The launch's wait limit (DasParams::waitLimitNs, 0 = kWaitLimitNs).
__device__ __forceinline__ uint64_t wait_limit(const DasParams& p)
{
	return p.waitLimitNs ? p.waitLimitNs : kWaitLimitNs;
}

template<bool ANALYTIC, int S> struct Sample;
template<int S> struct Sample<true, S> {
	using T = typename Complex<S>::T;
	static constexpr bool kAnalytic = true;
	static constexpr int kAlign = 16 / static_cast<int>(sizeof(T));  // elements per 16 bytes
	static __device__ __forceinline__ float2 load(const T* s) { return Complex<S>::load(s); }
	static __device__ __forceinline__ void accumulate(const T* s, float k, float2& acc)
	{
		const float2 a = Complex<S>::load(s);
		const float2 b = Complex<S>::load(s + 1);
		const float w0 = 1.0f - k;
		acc.x = fmaf(w0, a.x, acc.x);
		acc.y = fmaf(w0, a.y, acc.y);
		acc.x = fmaf(k, b.x, acc.x);
		acc.y = fmaf(k, b.y, acc.y);
	}
};
template<int S> struct Sample<false, S> {
	using T = typename Real<S>::T;
	static constexpr bool kAnalytic = false;
	static constexpr int kAlign = 16 / static_cast<int>(sizeof(T));
	static __device__ __forceinline__ void accumulate(const T* s, float k, float2& acc)
	{
		acc.x = fmaf(1.0f - k, Real<S>::load(s), acc.x);
		acc.x = fmaf(k, Real<S>::load(s + 1), acc.x);
	}
};

// ----------------------------------------------------------------- delays
// FP32 tiles: delay d = fl(txd + rxd) as in the reference; floor(d) by one
// round-down add against 2^23 (split_delay of the plain kernel): every d
// outside [0, 2^23) gives an index the unsigned range test rejects.
//
// FP64 tiles: the per-pixel transmit and receive delays are computed in
// double and stored as int32 fixed point with F fractional bits, F chosen per
// tile so that every term stays below 2^30 in magnitude (a sum never
// overflows): F = 30 - ceil(log2(largest |term| + 2)), at most 20 (2^-20
// sample) and at least 9 for delays up to 2^21 samples. A gather adds the two
// integers, idx = q >> F (floor, negative for negative delays) and k = the
// low F bits / 2^F, both exact.
struct Fixed {
	int F;           // fractional bits
	int mask;        // 2^F - 1
	int shift;       // 23 - F: places the fraction in a float mantissa
	double scale;    // 2^F
};

__device__ __forceinline__ Fixed fixed_format(float largest)
{
	const int e = ((__float_as_int(largest + 2.0f) >> 23) & 0xff) - 126;  // largest + 2 < 2^e
	Fixed f;
	f.F = max(9, min(20, 30 - e));
	f.mask = (1 << f.F) - 1;
	f.shift = 23 - f.F;
	f.scale = static_cast<double>(1 << f.F);
	return f;
}

__device__ __forceinline__ int split_delay(float d, float& k)
{
	const float t0 = __fadd_rd(d, 8388608.0f);
	k = d - (t0 - 8388608.0f);
	return static_cast<int>(__float_as_uint(t0) - 0x4B000000u);
}

__device__ __forceinline__ float to_fixed(double tau, const Fixed& f)
{
	return __int_as_float(__double2int_rn(fmin(fmax(tau * f.scale, -1073741823.0), 1073741823.0)));
}

__device__ __forceinline__ double distance3d_z0_f64(float ex, float ey, float px, float py, float pz)
{
	const double dx = static_cast<double>(px) - ex;
	const double dy = static_cast<double>(py) - ey;
	const double dz = pz;
	return sqrt(dx * dx + dy * dy + dz * dz);
}

template<bool Q> struct Delay;
template<> struct Delay<false> {
	static __device__ __forceinline__ int split(float txv, float rxv, float& k, const Fixed&)
	{
		return split_delay(__fadd_rn(txv, rxv), k);
	}
	static __device__ __forceinline__ float rx(const DasParams& p, float4 e, float px, float py, float pz,
			const Fixed&)
	{
		return __fmul_rn(distance3d_z0(e.x, e.y, px, py, pz), p.invCT);
	}
	static __device__ __forceinline__ float tx(const DasParams& p, float2 e, float px, float py, float pz,
			const Fixed&)
	{
		return __fadd_rn(p.signalOffset, __fmul_rn(distance3d_z0(e.x, e.y, px, py, pz), p.invCT));
	}
};
template<> struct Delay<true> {
	static __device__ __forceinline__ int split(float txv, float rxv, float& k, const Fixed& f)
	{
		const int q = __float_as_int(txv) + __float_as_int(rxv);
		k = __int_as_float(0x3F800000 | ((q & f.mask) << f.shift)) - 1.0f;
		return q >> f.F;
	}
	static __device__ __forceinline__ float rx(const DasParams& p, float4 e, float px, float py, float pz,
			const Fixed& f)
	{
		return to_fixed(distance3d_z0_f64(e.x, e.y, px, py, pz) * p.invCTd, f);
	}
	static __device__ __forceinline__ float tx(const DasParams& p, float2 e, float px, float py, float pz,
			const Fixed& f)
	{
		return to_fixed(p.signalOffsetd + distance3d_z0_f64(e.x, e.y, px, py, pz) * p.invCTd, f);
	}
};

// Contribution of one staged (or empty) window to one grid point:
// acc += (1-k) s[idx] + k s[idx+1]. Every delay of the tile lies inside its
// window, so the range test alone guards the stage read; an empty window
// rejects every index. Branch-free: an index out of range reads both taps
// from the zero slot with k = 0 (adds exactly 0, whatever the delay was).
template<typename SP, bool Q>
__device__ __forceinline__ void gather_staged(const typename SP::T* buf, int base, float txv, float rxv,
		unsigned lastIdx, const Fixed& fx, const typename SP::T* zero, float2& acc)
{
	float k;
	const int i = Delay<Q>::split(txv, rxv, k, fx);
	const bool ok = static_cast<unsigned>(i) <= lastIdx;
	const typename SP::T* src = ok ? buf + (i + base) : zero;
	SP::accumulate(src, ok ? k : 0.0f, acc);
}

// A window gathered from global memory (`src` = the A-scan).
template<typename SP, bool Q>
__device__ __forceinline__ void gather_global(const typename SP::T* src, float txv, float rxv, unsigned lastIdx,
		const Fixed& fx, float2& acc)
{
	float k;
	const int i = Delay<Q>::split(txv, rxv, k, fx);
	if (static_cast<unsigned>(i) <= lastIdx) SP::accumulate(src + i, k, acc);
}

// Any window kind: staged, empty, or gathered from global memory.
template<typename SP, bool Q>
__device__ __forceinline__ void gather_any(int4 wm, const typename SP::T* buf, const typename SP::T* sig,
		size_t txStride, unsigned r, size_t sigStride, float txv, float rxv, unsigned lastIdx, const Fixed& fx,
		float2& acc)
{
	float k;
	const int i = Delay<Q>::split(txv, rxv, k, fx);
	if (static_cast<unsigned>(i) <= lastIdx) {
		if (wm.z >= 0) {
			SP::accumulate(buf + (i + wm.y), k, acc);
		} else if (wm.z == kGlobalWindow) {
			SP::accumulate(sig + wm.w * txStride + static_cast<size_t>(r) * sigStride + i, k, acc);
		}
	}
}


}  // namespace tile
}  // namespace usgb
