// Staged delay-and-sum: one thread block per tile of 32 columns x TROWS rows
// of grid points; per (tx, rx) pair, the window of the A-scan that the tile's
// delays can reach is copied into shared memory by a producer warp with bulk
// copies (cp.async.bulk, completion on an mbarrier), several windows per
// pipeline stage, and the consumer warps gather both interpolation taps from
// shared memory.
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
//
// The per-tile body is a device function that keeps the pipeline's stage
// counter across calls, so one persistent block can run tiles of many frames
// back to back (batched kernel): the barriers are initialised once and their
// phases simply continue.
#include <cuda_runtime.h>

#include "usgb_common.cuh"
#include "usgb_das_cf.cuh"
#include "usgb_das_tile.cuh"
#include "usgb_internal.h"

namespace usgb {

namespace {

using namespace tile;

constexpr int kMaxWindows = 32;     // windows per stage (one per producer lane)

// One stage: up to 32 windows of consecutive transmitters of one receiver.
// Window w is (txd byte offset t * P * 4, base, kind, t): sample idx of a
// staged window sits at stage element idx + base; kind is kGlobalWindow or
// kEmptyWindow for windows that carry no bytes, else 0.
struct StageMeta {
	int count;
	int lastOfRx;   // the stage ends its receiver
	int firstOdd;   // its first transmitter is odd
	int anyGlobal;  // some window is gathered from global memory
	int4 win[kMaxWindows];
};

// Shared-memory layout (byte offsets), computed identically on host and
// device, for at most maxTx / maxRx elements.
struct StagedLayout {
	unsigned bars, tileMax, zero, meta, rxinfo, minmax, partial, txd, stage, total;
	__host__ __device__ StagedLayout(unsigned maxTx, unsigned maxRx, unsigned trows, unsigned capBytes, unsigned stages)
	{
		bars = 0;
		tileMax = 2 * stages * 8;
		zero = (tileMax + 8 + 15) & ~15u;
		meta = zero + 16;
		rxinfo = meta + stages * static_cast<unsigned>(sizeof(StageMeta));
		rxinfo = (rxinfo + 15) & ~15u;
		minmax = rxinfo + maxRx * 16;
		partial = minmax + 2 * (maxTx + maxRx) * 4;
		txd = partial + 2 * trows * (maxTx + maxRx) * 4;
		txd = (txd + 15) & ~15u;
		stage = txd + maxTx * 32 * trows * 4;
		stage = (stage + 127) & ~127u;
		total = stage + stages * capBytes;
	}
};

// Pointers into the block's shared memory.
struct Smem {
	uint64_t* full;
	uint64_t* empty;
	int* tileMax;    // [2]: largest transmit / receive delay of the tile (bits of a float >= 0)
	const unsigned char* zero;  // 16 zero bytes: the two taps of a gather that is out of range
	StageMeta* meta;
	float* minT;     // [maxTx]
	float* maxT;     // [maxTx]
	float* minR;     // [maxRx]
	float* maxR;     // [maxRx]
	float4* rxinfo;  // [maxRx]: receiver (x, y, apodization / storage scale, 0)
	float* partMin;  // [TROWS][maxTx + maxRx]
	float* partMax;
	float* txd;      // [maxTx][P]: FP32 delays, or fixed-point delays (int bits) in an FP64 tile
	unsigned char* stageBuf;
	unsigned nst;
	unsigned capBytes;
	unsigned maxE;   // maxTx + maxRx (row stride of the partial arrays)
};

__device__ __forceinline__ Smem carve(unsigned char* smem, const StagedLayout& lay, unsigned maxTx, unsigned maxRx,
		unsigned trows, unsigned nst, unsigned capBytes)
{
	Smem s;
	s.full = reinterpret_cast<uint64_t*>(smem + lay.bars);
	s.empty = s.full + nst;
	s.tileMax = reinterpret_cast<int*>(smem + lay.tileMax);
	s.zero = smem + lay.zero;
	s.meta = reinterpret_cast<StageMeta*>(smem + lay.meta);
	s.rxinfo = reinterpret_cast<float4*>(smem + lay.rxinfo);
	s.minT = reinterpret_cast<float*>(smem + lay.minmax);
	s.maxT = s.minT + maxTx;
	s.minR = s.maxT + maxTx;
	s.maxR = s.minR + maxRx;
	s.partMin = reinterpret_cast<float*>(smem + lay.partial);
	s.partMax = s.partMin + trows * (maxTx + maxRx);
	s.txd = reinterpret_cast<float*>(smem + lay.txd);
	s.stageBuf = smem + lay.stage;
	s.nst = nst;
	s.capBytes = capBytes;
	s.maxE = maxTx + maxRx;
	return s;
}

__device__ __forceinline__ void init_barriers(const Smem& sm, int trows)
{
	if (threadIdx.x < 4) reinterpret_cast<unsigned*>(const_cast<unsigned char*>(sm.zero))[threadIdx.x] = 0u;
	if (threadIdx.x == 0) {
		for (unsigned s = 0; s < sm.nst; ++s) {
			mbar_init(&sm.full[s], 1);
			mbar_init(&sm.empty[s], trows);
		}
		fence_barrier_init();
	}
	__syncthreads();
}

// ------------------------------------------------------------- producer
// The 32 lanes size 32 consecutive transmit windows of the current receiver
// at once; a prefix sum packs as many as fit into the stage, lane 0 arms the
// stage's barrier with the total byte count and every lane issues its own
// bulk copy. `margin` widens every window (FP64 tiles: their delays may sit
// a fraction of a sample outside the FP32 bounds the windows come from).
template<typename SP, int TROWS>
__device__ bool produce(const DasParams& p, const Smem& sm, int& it, float margin)
{
	using T = typename SP::T;
	constexpr int P = 32 * TROWS;
	const int nst = static_cast<int>(sm.nst);
	const unsigned capBytes = sm.capBytes;
	const int lane = threadIdx.x & 31;
	const int L = static_cast<int>(p.L);
	const size_t txStride = static_cast<size_t>(p.numRx) * p.sigStride;
	const T* sig = reinterpret_cast<const T*>(p.sig);
	const int itStart = it;
	// Ring slot and phase of stage `it`, carried along (no division per stage).
	int s = it % nst;
	unsigned phase = static_cast<unsigned>(it / nst) & 1u;
	bool ok = true;
	for (unsigned r = 0; r < p.numRx && ok; ++r) {
		unsigned t0 = 0;
		while (t0 < p.numTx) {
			if (it >= nst) {
				bool w = true;
				if (lane == 0) w = mbar_wait_bounded(&sm.empty[s], phase ^ 1u, wait_limit(p));
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
				const float a = __fadd_rn(sm.minT[t], sm.minR[r]);
				const float b = __fadd_rn(sm.maxT[t], sm.maxR[r]);
				// Window [lo, hi] of sample indices (a valid gather reads idx and idx + 1).
				const float lof = fmaxf(floorf(a) - margin, 0.0f);
				const float hif = fminf(floorf(b) + 1.0f + margin, static_cast<float>(L - 1));
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
			const bool anyGlobal = __ballot_sync(0xffffffffu, fits && kind == kGlobalWindow) != 0u;
			const unsigned total = __shfl_sync(0xffffffffu, incl, n - 1);
			const unsigned excl = incl - wb;
			StageMeta& m = sm.meta[s];
			if (lane < n) {
				const int base = (kind == 0) ? static_cast<int>(excl / sizeof(T)) - lo : 0;
				m.win[lane] = make_int4(static_cast<int>(t * (P * 4u)), base, kind, static_cast<int>(t));
			}
			if (lane == 0) {
				m.count = n;
				m.lastOfRx = (t0 + n == p.numTx) ? 1 : 0;
				m.firstOdd = static_cast<int>(t0 & 1u);
				m.anyGlobal = anyGlobal ? 1 : 0;
			}
			__threadfence_block();
			__syncwarp();
			// The test hook leaves this stage unarmed: its consumers' wait runs out.
			const bool skip = p.testSkipStage != 0u && it - itStart + 1 == static_cast<int>(p.testSkipStage);
			if (lane == 0 && !skip) mbar_arrive_expect_tx(&sm.full[s], total);
			__syncwarp();
			if (lane < n && wb > 0 && !skip) {
				const T* src = sig + t * txStride + static_cast<size_t>(r) * p.sigStride + lo;
				bulk_copy_g2s(sm.stageBuf + static_cast<size_t>(s) * capBytes + excl, src, wb, &sm.full[s]);
			}
			t0 += static_cast<unsigned>(n);
			++it;
			if (++s == nst) {
				s = 0;
				phase ^= 1u;
			}
		}
	}
	// Let this tile's last copies land before the block moves on or exits:
	// every stage still in the ring is waited for, also after one of them
	// gave up (a stage that was never armed), so no copy is left in flight.
	if (lane == 0) {
		const int from = (it - nst > itStart) ? it - nst : itStart;
		for (int j = from; j < it; ++j) {
			if (!mbar_wait_bounded(&sm.full[j % nst], (j / nst) & 1, wait_limit(p))) {
				atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
				ok = false;
			}
		}
	}
	return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

// ------------------------------------------------------------- consumers
// Receiver-major: per receiver, every staged window (one per transmitter) of
// the grid point; its even / odd transmitter terms go to two accumulators.
template<typename SP, int CF, int TROWS, bool Q>
__device__ bool consume(const DasParams& p, const Smem& sm, int& it, float px, float py, float pz, bool active,
		unsigned pix, const Fixed& fx)
{
	using T = typename SP::T;
	const int nst = static_cast<int>(sm.nst);
	const unsigned capBytes = sm.capBytes;
	const int slot = threadIdx.x;
	const unsigned lastIdx = p.L - 2;
	const size_t txStride = static_cast<size_t>(p.numRx) * p.sigStride;
	const T* sig = reinterpret_cast<const T*>(p.sig);
	const char* txdSlot = reinterpret_cast<const char*>(sm.txd + slot);
	const T* zero = reinterpret_cast<const T*>(sm.zero);
	float2 total = make_float2(0.f, 0.f);
	CFState<CF> cf;
	float2 acc = make_float2(0.f, 0.f);  // receiver r's terms, in transmitter order
	unsigned r = 0;
	// Receiver r's delay, and the next receiver's computed one receiver
	// ahead (its latency hides behind the current receiver's gathers).
	float rxd = Delay<Q>::rx(p, sm.rxinfo[0], px, py, pz, fx);
	float rxdNext = (p.numRx > 1) ? Delay<Q>::rx(p, sm.rxinfo[1], px, py, pz, fx) : 0.0f;
	// Ring slot and phase of stage `it`, carried along (no division per stage).
	int s = it % nst;
	unsigned phase = static_cast<unsigned>(it / nst) & 1u;
	while (r < p.numRx) {
		if (!mbar_wait_bounded(&sm.full[s], phase, wait_limit(p))) {
			atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
			return false;
		}
		const StageMeta& m = sm.meta[s];
		const T* buf = reinterpret_cast<const T*>(sm.stageBuf + static_cast<size_t>(s) * capBytes);
		const int4 head = *reinterpret_cast<const int4*>(&m.count);
		const int n = head.x;
		// Windows of a stage are consecutive transmitters of receiver r.
		if (!head.w) {
			int w = 0;
#pragma unroll 2
			for (; w + 1 < n; w += 2) {
				const int2 wa = *reinterpret_cast<const int2*>(&m.win[w]);
				const int2 wb = *reinterpret_cast<const int2*>(&m.win[w + 1]);
				gather_staged<SP, Q>(buf, wa.y, *reinterpret_cast<const float*>(txdSlot + wa.x), rxd, lastIdx, fx, zero, acc);
				gather_staged<SP, Q>(buf, wb.y, *reinterpret_cast<const float*>(txdSlot + wb.x), rxd, lastIdx, fx, zero, acc);
			}
			if (w < n) {
				const int2 wa = *reinterpret_cast<const int2*>(&m.win[w]);
				gather_staged<SP, Q>(buf, wa.y, *reinterpret_cast<const float*>(txdSlot + wa.x), rxd, lastIdx, fx, zero, acc);
			}
		} else {
			for (int w = 0; w < n; ++w) {
				const int4 wa = m.win[w];
				const float txv = *reinterpret_cast<const float*>(txdSlot + wa.x);
				gather_any<SP, Q>(wa, buf, sig, txStride, r, p.sigStride, txv, rxd, lastIdx, fx, acc);
			}
		}
		const int last = head.y;
		__syncwarp();
		if ((threadIdx.x & 31) == 0) mbar_arrive(&sm.empty[s]);
		++it;
		if (++s == nst) {
			s = 0;
			phase ^= 1u;
		}
		if (last) {
			const float2 rs = receiver_sum(acc, sm.rxinfo[r].z);
			total.x += rs.x;
			total.y += rs.y;
			cf.add(rs);
			acc = make_float2(0.f, 0.f);
			++r;
			rxd = rxdNext;
			if (r + 1 < p.numRx) rxdNext = Delay<Q>::rx(p, sm.rxinfo[r + 1], px, py, pz, fx);
		}
	}
	if (active) {
		const float v = SP::kAnalytic ? magnitude(total) : total.x;
		p.value[pix] = v * p.valueCoef;
		p.factor[pix] = cf.result(p.numRx, p, total);
	}
	return true;
}

// One tile (bx, by) of one frame. `it` is the block's running stage counter
// (the same value in every thread on entry and on exit). Returns false after a
// wait gave up (the error is recorded in p.errWord).
template<int S, int CF, bool ANALYTIC, int TROWS>
__device__ bool staged_tile(const DasParams& p, const Smem& sm, unsigned bx, unsigned by, int& it)
{
	using SP = Sample<ANALYTIC, S>;
	constexpr int P = 32 * TROWS;
	const int warp = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;
	const bool producer = warp == TROWS;
	const unsigned col = bx * 32 + lane;
	const unsigned row = by * TROWS + warp;
	const bool active = !producer && col < p.ncols && row < p.nrows;
	const unsigned pix = col * p.nrows + row;
	const int slot = warp * 32 + lane;
	const unsigned nE = p.numTx + p.numRx;

	// A consumer thread beyond the grid's edge takes the delays of the
	// nearest grid point of its tile (and stores nothing), so that every
	// consumer delay lies inside every window of the tile.
	float px = 0.f, py = 0.f, pz = 0.f;
	if (!producer) {
		const unsigned q = min(col, p.ncols - 1) * p.nrows + min(row, p.nrows - 1);
		px = p.grid[3 * q];
		py = p.grid[3 * q + 1];
		pz = p.grid[3 * q + 2];
	}
	if (threadIdx.x == 0) {
		sm.tileMax[0] = 0;
		sm.tileMax[1] = 0;
	}
	for (unsigned r = threadIdx.x; r < p.numRx; r += blockDim.x) {
		sm.rxinfo[r] = make_float4(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), __ldg(&p.apod[r]) * p.invScale, 0.f);
	}
	// FP32 transmit-delay table and per-warp min/max of every element's delay.
	if (!producer) {
		for (unsigned e = 0; e < nE; ++e) {
			float v;
			if (e < p.numTx) {
				const float dist = distance3d_z0(__ldg(&p.txXY[2 * e]), __ldg(&p.txXY[2 * e + 1]), px, py, pz);
				v = __fadd_rn(p.signalOffset, __fmul_rn(dist, p.invCT));
				sm.txd[e * P + slot] = v;
			} else {
				const unsigned r = e - p.numTx;
				v = __fmul_rn(distance3d_z0(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), px, py, pz), p.invCT);
			}
			float mn = v, mx = v;
			for (int o = 16; o > 0; o >>= 1) {
				mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
				mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
			}
			if (lane == 0) {
				sm.partMin[warp * sm.maxE + e] = mn;
				sm.partMax[warp * sm.maxE + e] = mx;
			}
		}
	}
	__syncthreads();
	float topT = 0.f, topR = 0.f;
	for (unsigned e = threadIdx.x; e < nE; e += blockDim.x) {
		float mn = sm.partMin[e], mx = sm.partMax[e];
		for (int w = 1; w < TROWS; ++w) {
			mn = fminf(mn, sm.partMin[w * sm.maxE + e]);
			mx = fmaxf(mx, sm.partMax[w * sm.maxE + e]);
		}
		if (e < p.numTx) { sm.minT[e] = mn; sm.maxT[e] = mx; topT = fmaxf(topT, mx); }
		else { sm.minR[e - p.numTx] = mn; sm.maxR[e - p.numTx] = mx; topR = fmaxf(topR, mx); }
	}
	// Non-negative floats order like their bit patterns.
	if (topT > 0.f) atomicMax(&sm.tileMax[0], __float_as_int(topT));
	if (topR > 0.f) atomicMax(&sm.tileMax[1], __float_as_int(topR));
	__syncthreads();

	// FP64 geometry where the FP32 delays could be off by more than 1/64
	// sample: the tile's largest delay is above kDeepDelaySamples.
	const float topTx = __int_as_float(sm.tileMax[0]), topRx = __int_as_float(sm.tileMax[1]);
	const bool q = p.delayMode == 2 || (p.delayMode == 0 && topTx + topRx > kDeepDelaySamples);
	const Fixed fx = fixed_format(fmaxf(fmaxf(topTx, topRx), fabsf(p.signalOffset)));
	if (q && !producer) {
		// Each thread replaces only its own column of the table.
		for (unsigned t = 0; t < p.numTx; ++t) {
			const double dist = distance3d_z0_f64(__ldg(&p.txXY[2 * t]), __ldg(&p.txXY[2 * t + 1]), px, py, pz);
			sm.txd[t * P + slot] = to_fixed(p.signalOffsetd + dist * p.invCTd, fx);
		}
	}
	if (producer) return produce<SP, TROWS>(p, sm, it, q ? 2.0f : 0.0f);
	return q ? consume<SP, CF, TROWS, true>(p, sm, it, px, py, pz, active, pix, fx)
	         : consume<SP, CF, TROWS, false>(p, sm, it, px, py, pz, active, pix, fx);
}

// Single frame: one block per tile.
template<int S, int CF, bool ANALYTIC, int TROWS>
__global__ void __launch_bounds__((TROWS + 1) * 32, 1)
das_staged_kernel(DasParams p)
{
	extern __shared__ __align__(128) unsigned char smem[];
	const StagedLayout lay(p.numTx, p.numRx, TROWS, p.stageBytes, p.stages);
	const Smem sm = carve(smem, lay, p.numTx, p.numRx, TROWS, p.stages, p.stageBytes);
	init_barriers(sm, TROWS);
	int it = 0;
	staged_tile<S, CF, ANALYTIC, TROWS>(p, sm, blockIdx.x, blockIdx.y, it);
}

template<int S, bool ANALYTIC, int TROWS>
__device__ __forceinline__ bool tile_any_cf(const DasParams& p, int cf, const Smem& sm, unsigned bx, unsigned by, int& it)
{
	if (!ANALYTIC) {
		return (cf == CF_SCF) ? staged_tile<S, CF_SCF, false, TROWS>(p, sm, bx, by, it)
		                      : staged_tile<S, CF_NONE, false, TROWS>(p, sm, bx, by, it);
	}
	switch (cf) {
	case CF_PCF: return staged_tile<S, CF_PCF, true, TROWS>(p, sm, bx, by, it);
	case CF_SCF: return staged_tile<S, CF_SCF, true, TROWS>(p, sm, bx, by, it);
	case CF_MF: return staged_tile<S, CF_MF, true, TROWS>(p, sm, bx, by, it);
	default: return staged_tile<S, CF_NONE, true, TROWS>(p, sm, bx, by, it);
	}
}

// Many frames: persistent blocks walk the tiles of every frame in the batch
// (frames of different sizes and coherence factors; same storage type).
template<int S, bool ANALYTIC, int TROWS>
__global__ void __launch_bounds__((TROWS + 1) * 32, 1)
das_staged_batch_kernel(const BatchDasFrame* __restrict__ frames, const BatchHeader* __restrict__ hdr,
		unsigned maxTx, unsigned maxRx, unsigned capBytes, unsigned stages)
{
	extern __shared__ __align__(128) unsigned char smem[];
	__shared__ DasParams sp;
	__shared__ int sAbort;
	const StagedLayout lay(maxTx, maxRx, TROWS, capBytes, stages);
	const Smem sm = carve(smem, lay, maxTx, maxRx, TROWS, stages, capBytes);
	if (threadIdx.x == 0) sAbort = 0;
	init_barriers(sm, TROWS);
	const unsigned count = hdr->count;
	const unsigned totalTiles = hdr->totalTiles;
	int it = 0;
	unsigned f = 0;
	for (unsigned w = blockIdx.x; w < totalTiles; w += gridDim.x) {
		while (f + 1 < count && frames[f + 1].tileBegin <= w) ++f;  // work items are visited in increasing order
		__syncthreads();  // the previous tile is done with sp and the shared tables
		if (threadIdx.x == 0) sp = frames[f].das;
		__syncthreads();
		if (sAbort) break;
		const unsigned local = w - frames[f].tileBegin;
		const unsigned tilesX = frames[f].tilesX;
		const bool ok = tile_any_cf<S, ANALYTIC, TROWS>(sp, frames[f].cf, sm, local % tilesX, local / tilesX, it);
		if (!ok) sAbort = 1;
	}
}

template<int S, int CF, bool ANALYTIC, int TROWS>
cudaError_t launch_one(const DasParams& p, cudaStream_t stream)
{
	const StagedLayout lay(p.numTx, p.numRx, TROWS, p.stageBytes, p.stages);
	cudaError_t e = cudaFuncSetAttribute(das_staged_kernel<S, CF, ANALYTIC, TROWS>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lay.total));
	if (e != cudaSuccess) return e;
	const dim3 grid((p.ncols + 31) / 32, (p.nrows + TROWS - 1) / TROWS);
	das_staged_kernel<S, CF, ANALYTIC, TROWS><<<grid, (TROWS + 1) * 32, lay.total, stream>>>(p);
	return cudaGetLastError();
}

template<int S, int CF, bool ANALYTIC>
cudaError_t launch_rows(const DasParams& p, cudaStream_t stream)
{
	switch (p.tileRows) {
	case 4: return launch_one<S, CF, ANALYTIC, 4>(p, stream);
	case 16: return launch_one<S, CF, ANALYTIC, 16>(p, stream);
	default: return launch_one<S, CF, ANALYTIC, 8>(p, stream);
	}
}

template<int S>
cudaError_t dispatch(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	if (!analytic) {
		return (cf == CF_SCF) ? launch_rows<S, CF_SCF, false>(p, stream) : launch_rows<S, CF_NONE, false>(p, stream);
	}
	switch (cf) {
	case CF_PCF: return launch_rows<S, CF_PCF, true>(p, stream);
	case CF_SCF: return launch_rows<S, CF_SCF, true>(p, stream);
	case CF_MF: return launch_rows<S, CF_MF, true>(p, stream);
	default: return launch_rows<S, CF_NONE, true>(p, stream);
	}
}

template<int S, bool ANALYTIC, int TROWS>
cudaError_t launch_batch_one(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		cudaStream_t stream)
{
	const StagedLayout lay(c.maxTx, c.maxRx, TROWS, c.stageBytes, c.stages);
	cudaError_t e = cudaFuncSetAttribute(das_staged_batch_kernel<S, ANALYTIC, TROWS>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lay.total));
	if (e != cudaSuccess) return e;
	das_staged_batch_kernel<S, ANALYTIC, TROWS><<<c.blocks, (TROWS + 1) * 32, lay.total, stream>>>(
			frames, hdr, c.maxTx, c.maxRx, c.stageBytes, c.stages);
	return cudaGetLastError();
}

template<int S, bool ANALYTIC>
cudaError_t batch_rows(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c, cudaStream_t stream)
{
	switch (c.tileRows) {
	case 4: return launch_batch_one<S, ANALYTIC, 4>(frames, hdr, c, stream);
	case 16: return launch_batch_one<S, ANALYTIC, 16>(frames, hdr, c, stream);
	default: return launch_batch_one<S, ANALYTIC, 8>(frames, hdr, c, stream);
	}
}

}  // namespace

size_t das_staged_smem_bytes(unsigned numTx, unsigned numRx, unsigned tileRows, unsigned capBytes, unsigned stages)
{
	return StagedLayout(numTx, numRx, tileRows, capBytes, stages).total;
}

cudaError_t launch_das_staged(const DasParams& p, int storage, int cf, bool analytic, cudaStream_t stream)
{
	switch (storage) {
	case STORE_F16: return dispatch<STORE_F16>(p, cf, analytic, stream);
	case STORE_BF16: return dispatch<STORE_BF16>(p, cf, analytic, stream);
	default: return dispatch<STORE_F32>(p, cf, analytic, stream);
	}
}

cudaError_t launch_das_staged_batch(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		int storage, bool analytic, cudaStream_t stream)
{
	if (analytic) {
		switch (storage) {
		case STORE_F16: return batch_rows<STORE_F16, true>(frames, hdr, c, stream);
		case STORE_BF16: return batch_rows<STORE_BF16, true>(frames, hdr, c, stream);
		default: return batch_rows<STORE_F32, true>(frames, hdr, c, stream);
		}
	}
	switch (storage) {
	case STORE_F16: return batch_rows<STORE_F16, false>(frames, hdr, c, stream);
	case STORE_BF16: return batch_rows<STORE_BF16, false>(frames, hdr, c, stream);
	default: return batch_rows<STORE_F32, false>(frames, hdr, c, stream);
	}
}

}  // namespace usgb
