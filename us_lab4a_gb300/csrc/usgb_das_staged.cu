// Staged delay-and-sum kernel: one thread block per tile of 32 columns x
// TROWS rows of grid points; per (tx, rx) pair, the window of the A-scan that
// the tile's delays can reach is copied into shared memory by a producer warp
// with bulk copies (cp.async.bulk, completion on an mbarrier), several
// windows per pipeline stage, and the consumer warps gather both
// interpolation taps from shared memory.
//
// Arithmetic follows the plain kernel (usgb_das.cu) exactly: same delay
// rounding, same receiver-major accumulation, same coherence factors.
//
// Window bounds: for grid points p of the tile, delay(p) =
// fl(txd(p) + rxd(p)) with txd = fl(offset + fl(dist * invCT)). Rounded
// addition is monotonic in each argument, so floor(delay(p)) lies in
// [floor(fl(min txd + min rxd)), floor(fl(max txd + max rxd))], and every
// sample a valid gather reads (index and index + 1) lies in the window
// [lo, hi + 1] clipped to [0, L - 1].
//
// Warp layout: lane = column, warp = row; neighbouring columns have close
// delays, so the shared-memory gathers of a warp mostly hit the same or
// consecutive words.
#include <cuda_runtime.h>

#include "usgb_common.cuh"
#include "usgb_das_cf.cuh"
#include "usgb_internal.h"

namespace usgb {

namespace {

constexpr int kStages = 4;          // pipeline depth
constexpr int kMaxWindows = 32;     // windows per stage (one per producer lane)
constexpr int kGlobalWindow = -1;   // window too large for a stage: gather from global memory
constexpr int kEmptyWindow = -2;    // no valid sample can be reached
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

struct StageMeta {
	int count;
	int lastOfRx;
	int pad[2];
	int4 win[kMaxWindows];  // (tx, lo, off, 0) per window
};

// Shared-memory layout (byte offsets), computed identically on host and device.
struct StagedLayout {
	unsigned bars, meta, minmax, partial, txd, stage, total;
	unsigned capBytes;
	__host__ __device__ StagedLayout(unsigned numTx, unsigned numRx, unsigned trows, unsigned capBytes_)
	{
		capBytes = capBytes_;
		bars = 0;
		meta = 2 * kStages * 8;
		minmax = meta + kStages * static_cast<unsigned>(sizeof(StageMeta));
		minmax = (minmax + 15) & ~15u;
		partial = minmax + 2 * (numTx + numRx) * 4;
		txd = partial + 2 * trows * (numTx + numRx) * 4;
		txd = (txd + 15) & ~15u;
		stage = txd + numTx * 32 * trows * 4;
		stage = (stage + 127) & ~127u;
		total = stage + kStages * capBytes;
	}
};

template<bool ANALYTIC, int S> struct Sample;
template<int S> struct Sample<true, S> {
	using T = typename Complex<S>::T;
	static constexpr int kAlign = 16 / static_cast<int>(sizeof(T));  // elements per 16 bytes
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
	static constexpr int kAlign = 16 / static_cast<int>(sizeof(T));
	static __device__ __forceinline__ void accumulate(const T* s, float k, float2& acc)
	{
		acc.x = fmaf(1.0f - k, Real<S>::load(s), acc.x);
		acc.x = fmaf(k, Real<S>::load(s + 1), acc.x);
	}
};

__device__ __forceinline__ int floor_to_int(float v)
{
	return static_cast<int>(floorf(v));
}

template<int S, int CF, bool ANALYTIC, int TROWS>
__global__ void __launch_bounds__((TROWS + 1) * 32, 1)
das_staged_kernel(DasParams p, unsigned capBytes)
{
	using SP = Sample<ANALYTIC, S>;
	using T = typename SP::T;
	constexpr int P = 32 * TROWS;
	extern __shared__ __align__(128) unsigned char smem[];
	const StagedLayout lay(p.numTx, p.numRx, TROWS, capBytes);
	uint64_t* full = reinterpret_cast<uint64_t*>(smem + lay.bars);
	uint64_t* empty = full + kStages;
	StageMeta* meta = reinterpret_cast<StageMeta*>(smem + lay.meta);
	float* minT = reinterpret_cast<float*>(smem + lay.minmax);
	float* maxT = minT + p.numTx;
	float* minR = maxT + p.numTx;
	float* maxR = minR + p.numRx;
	float* partMin = reinterpret_cast<float*>(smem + lay.partial);          // [TROWS][numTx + numRx]
	float* partMax = partMin + TROWS * (p.numTx + p.numRx);
	float* txd = reinterpret_cast<float*>(smem + lay.txd);                  // [numTx][P]
	unsigned char* stageBuf = smem + lay.stage;

	const int warp = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;
	const bool producer = warp == TROWS;
	const unsigned col = blockIdx.x * 32 + lane;
	const unsigned row = blockIdx.y * TROWS + warp;
	const bool active = !producer && col < p.ncols && row < p.nrows;
	const unsigned pix = col * p.nrows + row;
	const int slot = warp * 32 + lane;
	const unsigned nE = p.numTx + p.numRx;

	float px = 0.f, py = 0.f, pz = 0.f;
	if (active) {
		px = p.grid[3 * pix];
		py = p.grid[3 * pix + 1];
		pz = p.grid[3 * pix + 2];
	}
	// Transmit-delay table and per-warp min/max of every element's delay.
	if (!producer) {
		for (unsigned e = 0; e < nE; ++e) {
			float v;
			if (e < p.numTx) {
				const float dist = distance3d_z0(__ldg(&p.txXY[2 * e]), __ldg(&p.txXY[2 * e + 1]), px, py, pz);
				v = __fadd_rn(p.signalOffset, __fmul_rn(dist, p.invCT));
				txd[e * P + slot] = v;
			} else {
				const unsigned r = e - p.numTx;
				v = __fmul_rn(distance3d_z0(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), px, py, pz), p.invCT);
			}
			float mn = active ? v : __int_as_float(0x7f800000);   // +inf
			float mx = active ? v : __int_as_float(0xff800000);   // -inf
			for (int o = 16; o > 0; o >>= 1) {
				mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
				mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
			}
			if (lane == 0) {
				partMin[warp * nE + e] = mn;
				partMax[warp * nE + e] = mx;
			}
		}
	}
	if (threadIdx.x == 0) {
		for (int s = 0; s < kStages; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], TROWS);
		}
		fence_barrier_init();
	}
	__syncthreads();
	for (unsigned e = threadIdx.x; e < nE; e += blockDim.x) {
		float mn = partMin[e], mx = partMax[e];
		for (int w = 1; w < TROWS; ++w) {
			mn = fminf(mn, partMin[w * nE + e]);
			mx = fmaxf(mx, partMax[w * nE + e]);
		}
		if (e < p.numTx) { minT[e] = mn; maxT[e] = mx; }
		else { minR[e - p.numTx] = mn; maxR[e - p.numTx] = mx; }
	}
	__syncthreads();

	const int L = static_cast<int>(p.L);
	const size_t txStride = static_cast<size_t>(p.numRx) * p.sigStride;
	const T* sig = reinterpret_cast<const T*>(p.sig);

	if (producer) {
		// -------------------------------------------------------------- producer
		// The 32 lanes size 32 consecutive transmit windows of the current
		// receiver at once; a prefix sum packs as many as fit into the stage,
		// lane 0 arms the stage's barrier with the total byte count and every
		// lane issues its own bulk copy.
		int it = 0;
		bool ok = true;
		for (unsigned r = 0; r < p.numRx && ok; ++r) {
			unsigned t0 = 0;
			while (t0 < p.numTx) {
				const int s = it % kStages;
				if (it >= kStages) {
					bool w = true;
					if (lane == 0) w = mbar_wait_bounded(&empty[s], ((it / kStages) - 1) & 1, kWaitLimitNs);
					w = __shfl_sync(0xffffffffu, w, 0);
					if (!w) {
						if (lane == 0) atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
						ok = false;
						break;
					}
				}
				const unsigned t = t0 + lane;
				int lo = 0, kind = kEmptyWindow;
				unsigned wb = 0;
				if (t < p.numTx) {
					const float a = __fadd_rn(minT[t], minR[r]);
					const float b = __fadd_rn(maxT[t], maxR[r]);
					// Window [lo, hi] of sample indices (a valid gather reads idx and idx + 1).
					const float lof = fmaxf(floorf(a), 0.0f);
					const float hif = fminf(floorf(b) + 1.0f, static_cast<float>(L - 1));
					if (lof <= static_cast<float>(L - 2) && hif >= 1.0f && hif >= lof) {
						lo = static_cast<int>(lof) & ~(SP::kAlign - 1);
						const unsigned cnt = static_cast<unsigned>(static_cast<int>(hif) - lo + 1);
						wb = (cnt * static_cast<unsigned>(sizeof(T)) + 15u) & ~15u;
						if (wb > capBytes) {  // larger than a whole stage: consumers read global memory
							kind = kGlobalWindow;
							wb = 0;
						} else {
							kind = 0;
						}
					}
				}
				unsigned incl = wb;
				for (int o = 1; o < 32; o <<= 1) {
					const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
					if (lane >= o) incl += v;
				}
				// Lanes that fit form a prefix (incl is non-decreasing); lane 0
				// always fits, since an oversized window carries no bytes.
				const bool fits = t < p.numTx && incl <= capBytes;
				const int n = __popc(__ballot_sync(0xffffffffu, fits));
				const unsigned total = __shfl_sync(0xffffffffu, incl, n - 1);
				const unsigned excl = incl - wb;
				StageMeta& m = meta[s];
				if (lane < n) {
					const int off = (kind == 0) ? static_cast<int>(excl / sizeof(T)) : kind;
					m.win[lane] = make_int4(static_cast<int>(t), lo, off, 0);
				}
				if (lane == 0) {
					m.count = n;
					m.lastOfRx = (t0 + n == p.numTx) ? 1 : 0;
				}
				__threadfence_block();
				__syncwarp();
				if (lane == 0) mbar_arrive_expect_tx(&full[s], total);
				__syncwarp();
				if (lane < n && wb > 0) {
					const T* src = sig + t * txStride + static_cast<size_t>(r) * p.sigStride + lo;
					bulk_copy_g2s(stageBuf + static_cast<size_t>(s) * capBytes + excl, src, wb, &full[s]);
				}
				t0 += static_cast<unsigned>(n);
				++it;
			}
		}
		// Let every issued copy land before the block can exit.
		if (lane == 0) {
			for (int j = (it > kStages ? it - kStages : 0); j < it; ++j) {
				if (!mbar_wait_bounded(&full[j % kStages], (j / kStages) & 1, kWaitLimitNs)) {
					atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
					break;
				}
			}
		}
		return;
	}

	// ------------------------------------------------------------------ consumers
	const unsigned lastIdx = static_cast<unsigned>(L - 2);
	float2 total = make_float2(0.f, 0.f);
	CFState<CF> cf;
	float2 acc = make_float2(0.f, 0.f);
	unsigned r = 0;
	float rxd = __fmul_rn(distance3d_z0(__ldg(&p.rxXY[0]), __ldg(&p.rxXY[1]), px, py, pz), p.invCT);
	int it = 0;
	bool ok = true;
	while (r < p.numRx) {
		const int s = it % kStages;
		if (!mbar_wait_bounded(&full[s], (it / kStages) & 1, kWaitLimitNs)) {
			atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
			ok = false;
			break;
		}
		const StageMeta& m = meta[s];
		const T* buf = reinterpret_cast<const T*>(stageBuf + static_cast<size_t>(s) * capBytes);
		const int n = m.count;
		for (int w = 0; w < n; ++w) {
			const int4 wm = m.win[w];
			const int t = wm.x;
			const int off = wm.z;
			const float d = fmaxf(__fadd_rn(txd[t * P + slot], rxd), -1.0f);
			const float t0 = __fadd_rd(d, 8388608.0f);
			const float k = d - (t0 - 8388608.0f);
			const int i = __float_as_int(t0) - 0x4B000000;
			if (active && static_cast<unsigned>(i) <= lastIdx) {
				if (off >= 0) {
					SP::accumulate(buf + (i - wm.y + off), k, acc);
				} else if (off == kGlobalWindow) {
					SP::accumulate(sig + t * txStride + static_cast<size_t>(r) * p.sigStride + i, k, acc);
				}
			}
		}
		const int last = m.lastOfRx;
		__syncwarp();
		if (lane == 0) mbar_arrive(&empty[s]);
		++it;
		if (last) {
			const float2 rs = receiver_sum(acc, __ldg(&p.apod[r]) * p.invScale);
			total.x += rs.x;
			total.y += rs.y;
			cf.add(rs);
			acc = make_float2(0.f, 0.f);
			++r;
			if (r < p.numRx) {
				rxd = __fmul_rn(distance3d_z0(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), px, py, pz), p.invCT);
			}
		}
	}
	if (ok && active) {
		const float v = ANALYTIC ? magnitude(total) : total.x;
		p.value[pix] = v * p.valueCoef;
		p.factor[pix] = cf.result(p.numRx, p, total);
	}
}

template<int S, int CF, bool ANALYTIC, int TROWS>
cudaError_t launch_one(const DasParams& p, unsigned capBytes, cudaStream_t stream)
{
	const StagedLayout lay(p.numTx, p.numRx, TROWS, capBytes);
	cudaError_t e = cudaFuncSetAttribute(das_staged_kernel<S, CF, ANALYTIC, TROWS>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lay.total));
	if (e != cudaSuccess) return e;
	const dim3 grid((p.ncols + 31) / 32, (p.nrows + TROWS - 1) / TROWS);
	das_staged_kernel<S, CF, ANALYTIC, TROWS><<<grid, (TROWS + 1) * 32, lay.total, stream>>>(p, capBytes);
	return cudaGetLastError();
}

template<int S, int CF, bool ANALYTIC>
cudaError_t launch_rows(const DasParams& p, unsigned capBytes, cudaStream_t stream)
{
	switch (p.tileRows) {
	case 4: return launch_one<S, CF, ANALYTIC, 4>(p, capBytes, stream);
	case 16: return launch_one<S, CF, ANALYTIC, 16>(p, capBytes, stream);
	default: return launch_one<S, CF, ANALYTIC, 8>(p, capBytes, stream);
	}
}

template<int S>
cudaError_t dispatch(const DasParams& p, int cf, bool analytic, unsigned capBytes, cudaStream_t stream)
{
	if (!analytic) {
		return (cf == CF_SCF) ? launch_rows<S, CF_SCF, false>(p, capBytes, stream)
		                      : launch_rows<S, CF_NONE, false>(p, capBytes, stream);
	}
	switch (cf) {
	case CF_PCF: return launch_rows<S, CF_PCF, true>(p, capBytes, stream);
	case CF_SCF: return launch_rows<S, CF_SCF, true>(p, capBytes, stream);
	case CF_MF: return launch_rows<S, CF_MF, true>(p, capBytes, stream);
	default: return launch_rows<S, CF_NONE, true>(p, capBytes, stream);
	}
}

}  // namespace

size_t das_staged_smem_bytes(unsigned numTx, unsigned numRx, unsigned tileRows, unsigned capBytes)
{
	return StagedLayout(numTx, numRx, tileRows, capBytes).total;
}

cudaError_t launch_das_staged(const DasParams& p, int storage, int cf, bool analytic, unsigned capBytes,
		cudaStream_t stream)
{
	switch (storage) {
	case STORE_F16: return dispatch<STORE_F16>(p, cf, analytic, capBytes, stream);
	case STORE_BF16: return dispatch<STORE_BF16>(p, cf, analytic, capBytes, stream);
	default: return dispatch<STORE_F32>(p, cf, analytic, capBytes, stream);
	}
}

}  // namespace usgb
