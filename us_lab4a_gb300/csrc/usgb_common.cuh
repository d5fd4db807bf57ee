// Shared device helpers of libusgb (STA/TFM delay-and-sum for GB300, sm_103a).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace usgb {

// Storage type of the prepared (analytic or real) signal tensor.
enum StorageKind : int { STORE_F32 = 0, STORE_F16 = 1, STORE_BF16 = 2 };

// Coherence factor selected per frame.
enum CFKind : int { CF_NONE = 0, CF_PCF = 1, CF_SCF = 2, CF_MF = 3 };

// Device-side error codes written to the context's error word.
enum DeviceError : unsigned { DEVERR_NONE = 0, DEVERR_WAIT_TIMEOUT = 1u, DEVERR_BAD_WINDOW = 2u };

// Complex sample codecs: a "pair" is one complex sample (re, im).
template<int S> struct Complex;
template<> struct Complex<STORE_F32> {
	using T = float2;
	static __device__ __forceinline__ float2 load(const T* p) { return *p; }
	static __device__ __forceinline__ T pack(float re, float im) { return make_float2(re, im); }
};
template<> struct Complex<STORE_F16> {
	using T = __half2;
	static __device__ __forceinline__ float2 load(const T* p) { return __half22float2(*p); }
	static __device__ __forceinline__ T pack(float re, float im) { return __floats2half2_rn(re, im); }
};
template<> struct Complex<STORE_BF16> {
	using T = __nv_bfloat162;
	static __device__ __forceinline__ float2 load(const T* p) { return __bfloat1622float2(*p); }
	static __device__ __forceinline__ T pack(float re, float im) { return __floats2bfloat162_rn(re, im); }
};

// Real sample codecs (real-RF path).
template<int S> struct Real;
template<> struct Real<STORE_F32> {
	using T = float;
	static __device__ __forceinline__ float load(const T* p) { return *p; }
	static __device__ __forceinline__ T pack(float v) { return v; }
};
template<> struct Real<STORE_F16> {
	using T = __half;
	static __device__ __forceinline__ float load(const T* p) { return __half2float(*p); }
	static __device__ __forceinline__ T pack(float v) { return __float2half_rn(v); }
};
template<> struct Real<STORE_BF16> {
	using T = __nv_bfloat16;
	static __device__ __forceinline__ float load(const T* p) { return __bfloat162float(*p); }
	static __device__ __forceinline__ T pack(float v) { return __float2bfloat16_rn(v); }
};

__device__ __forceinline__ uint64_t global_timer_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
	return t;
}

// Distance from an element at (ex, ey, 0) to a point (px, py, pz), without
// FMA contraction, so it rounds like the reference's
// std::sqrt(dx * dx + dy * dy + z * z) (src/util/Geometry.h:77-84; for
// ey = py = 0 it equals distance2DY0, src/util/Geometry.h:55-65).
__device__ __forceinline__ float distance3d_z0(float ex, float ey, float px, float py, float pz)
{
	const float dx = __fsub_rn(px, ex);
	const float dy = __fsub_rn(py, ey);
	const float s = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(pz, pz));
	return __fsqrt_rn(s);
}

}  // namespace usgb
