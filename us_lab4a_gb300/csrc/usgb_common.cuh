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

// ---------------------------------------------------------------------------
// Tensor memory (TMEM, 128 lanes x 512 columns of 32 bits per SM), inline
// PTX (tcgen05, sm_100a family). A warp reaches only the 32 lanes of its SM
// sub-partition (lanes 32 (warp % 4) .. + 31); an address is lane << 16 |
// column. Allocation and release are whole-warp operations of one warp of
// the block; the column count is a power of two in [32, 512].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
			:: "r"(smem_addr(dst)), "r"(ncols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
// Orders this thread's tensor-memory operations before (after) a barrier.
__device__ __forceinline__ void tmem_fence_before_sync()
{
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_after_sync()
{
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Eight consecutive columns of this thread's lane: store (complete when the
// call returns) and load (the values valid when the call returns).
__device__ __forceinline__ void tmem_store8(uint32_t taddr, const float (&v)[8])
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n\t"
			"tcgen05.wait::st.sync.aligned;"
			:: "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
			"r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
			"r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])) : "memory");
}
__device__ __forceinline__ void tmem_load8(uint32_t taddr, float (&v)[8])
{
	uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
			"tcgen05.wait::ld.sync.aligned;"
			: "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6), "=r"(r7)
			: "r"(taddr) : "memory");
	v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1); v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
	v[4] = __uint_as_float(r4); v[5] = __uint_as_float(r5); v[6] = __uint_as_float(r6); v[7] = __uint_as_float(r7);
}

// Bulk global -> shared copy completing on `bar` (both addresses 16-byte
// aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
			:: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

}  // namespace usgb
