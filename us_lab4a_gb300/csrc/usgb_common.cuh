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

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy (TMA, non-tensor) wrappers, inline PTX (sm_90+).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void fence_barrier_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
			:: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
	return ok != 0;
}

// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or about `hint_ns` nanoseconds pass, instead of spinning.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns) : "memory");
	return ok != 0;
}

// Bounded wait for the phase of `parity` to complete. Gives up after
// `limit_ns` nanoseconds and returns false; the caller records the error and
// winds down instead of waiting forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
	if (mbar_try_wait(bar, parity)) return true;
	const uint64_t t0 = global_timer_ns();
	for (;;) {
		if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
		if (global_timer_ns() - t0 > limit_ns) return false;
	}
}

// Orders this thread's earlier generic-proxy accesses of shared memory before
// the async-proxy (bulk copy) accesses it issues next.
__device__ __forceinline__ void fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk global -> shared copy completing on `bar` (both addresses 16-byte
// aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
			:: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

}  // namespace usgb
