// Receiver-group delay-and-sum: one thread block per tile of TCOLS (32 or
// 64) columns x TROWS rows of grid points (lane = column, TCOLS / 32 warps a
// row), like the staged kernel (usgb_das_staged.cu), but the pairs are
// visited receiver group by receiver group: for each group of kGroup
// receivers, every transmitter in turn, with the group's kGroup windows (one
// per receiver) staged together as one unit. A consumer thread keeps the group's receive delays and its kGroup
// receiver sums in registers and computes each transmitter's delay once per
// unit, so no per-pixel delay table lives in shared memory: a block holds
// only its stage ring and a few per-element tables, several blocks fit on an
// SM, and arrays of hundreds of elements (2D matrix probes) stage like small
// ones.
//
// Tile width: the delays change along a column by about 2 dz / (c / (fs U))
// samples per row (45 on cf2d) and little across columns, so a wider tile
// stages windows that are only a little longer for twice the points: 64 x 4
// tiles stage 12.2 GB per cf2d frame against 16.4 GB for 32 x 4, with half as
// many window copies, and one producer warp serves eight consumer warps;
// 64 x 8 tiles with stages of ~100 KiB (one block of 16 consumer warps per
// SM) stage 8.9 GB. Each stage is a barrier round trip gated by the slowest
// consumer warp, so fewer, larger stages run faster than deeper rings of
// small ones.
//
// Arithmetic is the plain kernel's, term for term: delay = fl(fl(offset +
// fl(dist_tx * invCT)) + fl(dist_rx * invCT)), the same index / fraction
// split, each receiver's terms summed in transmitter order into one
// accumulator, receivers folded into the total in order.
// Window bounds come from per-element min/max exactly as in the staged kernel;
// a window larger than stage_bytes / kGroup is gathered from global memory.
// FP64 geometry for deep tiles, bounded waits and the error word behave as in
// the staged kernel.
//
// This header holds the kernels; usgb_das_group_{f32,f16,bf16}.cu instantiate
// them for one storage type each (compiled in parallel) and usgb_das_group.cu
// dispatches.
#pragma once

#include <cuda_runtime.h>

#include "usgb_common.cuh"
#include "usgb_das_cf.cuh"
#include "usgb_das_tile.cuh"
#include "usgb_internal.h"

namespace usgb {

namespace {

using namespace tile;

constexpr int kGroup = 8;                  // receivers per group
constexpr int kMaxUnits = 32 / kGroup;     // units sized per producer pass (one lane per window)
// Unit flag: every window of the unit is staged whole, without clamping to
// the A-scan, so every delay of the tile for those pairs gives an index in
// [0, L - 2] and the gathers need no range test.
constexpr unsigned kUnitInterior = 0x100u;

// Block shape of a tile: NCW consumer warps and the producer. With two points
// per thread on 16 consumer warps (64 x 16 tiles) the consumers need more
// registers than an even share of the register file: the block then has
// 20 warps (5 warpgroups), launched at kLaunchRegs registers a thread; the
// producer warpgroup (the producer warp and 3 warps that exit) drops to
// kProducerRegs and the 4 consumer warpgroups rise to kConsumerRegs
// (setmaxnreg). The split fits the launch allocation:
// 128 x 64 + 512 x 104 = 61440 = 640 x 96 registers. Measured on the cf2d
// frame (64 x 16 tiles, 2 x 100 KiB stages): FP32 1.645 ms with 64 / 104,
// 1.659 ms without a split (17 warps at 96 registers, ~1 KB of spills), 1.82
// and 1.87 ms with the producer held to 40 and 32 registers (its spills
// slow the staging); FP16 1.12, 1.15, 1.08, 1.11 ms.
#ifndef USGB_GROUP_SPLIT
#define USGB_GROUP_SPLIT 1
#endif
#ifndef USGB_PRODUCER_REGS
#define USGB_PRODUCER_REGS 64
#endif
#ifndef USGB_CONSUMER_REGS
#define USGB_CONSUMER_REGS 104
#endif
// Single-frame kernels only: the split happens once per block, right before
// the producer and consumer paths part for good (batches loop over tiles, so
// the two paths would meet again and ptxas would hold both to the producer's
// count).
template<int NCW, int PY> struct GroupShape {
	static constexpr bool kSplit = USGB_GROUP_SPLIT && NCW == 16 && PY == 2;
	static constexpr int kWarps = kSplit ? NCW + 4 : NCW + 1;
	static constexpr int kLaunchRegs = 96;
	static constexpr int kProducerRegs = USGB_PRODUCER_REGS;
	static constexpr int kConsumerRegs = USGB_CONSUMER_REGS;
	static_assert(kProducerRegs % 8 == 0 && kConsumerRegs % 8 == 0 && kProducerRegs >= 24 && kConsumerRegs <= 256,
			"setmaxnreg counts are multiples of 8 in [24, 256]");
	static_assert(kProducerRegs <= kLaunchRegs && kConsumerRegs >= kLaunchRegs, "producer gives, consumers take");
	static_assert(!kSplit || 128 * kProducerRegs + NCW * 32 * kConsumerRegs <= kWarps * 32 * kLaunchRegs,
			"register split must fit in the launch allocation");
	static_assert(!kSplit || kWarps * 32 * kLaunchRegs <= 65536, "launch allocation exceeds the register file");
};

template<int N> __device__ __forceinline__ void regs_dec() { asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" :: "n"(N)); }
template<int N> __device__ __forceinline__ void regs_inc() { asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" :: "n"(N)); }


// One stage: up to kMaxUnits units (consecutive transmitters of one receiver
// group). Window j of unit u: sample idx of receiver g * kGroup + j sits at
// stage element idx + base[u][j].
struct GroupStage {
	int count;        // units in the stage
	int lastOfGroup;  // the stage ends its receiver group
	int anyGlobal;    // some window is gathered from global memory
	int pad;
	int2 unit[kMaxUnits];           // (transmitter, bit j set: window j from global memory; kUnitInterior)
	int base[kMaxUnits][kGroup];
};
static_assert(sizeof(GroupStage) % 16 == 0, "stage metadata must stay 16-byte aligned");

struct GroupLayout {
	unsigned bars, tileMax, zero, meta, rxinfo, txinfo, minmax, partial, stage, total;
	// cwarps: consumer warps (one per 32 points of the tile).
	__host__ __device__ GroupLayout(unsigned maxTx, unsigned maxRx, unsigned cwarps, unsigned capBytes, unsigned stages)
	{
		bars = 0;
		tileMax = 2 * stages * 8;
		zero = (tileMax + 8 + 15) & ~15u;
		meta = zero + 16;
		rxinfo = meta + stages * static_cast<unsigned>(sizeof(GroupStage));
		txinfo = rxinfo + maxRx * 16;
		minmax = (txinfo + maxTx * 8 + 15) & ~15u;
		partial = minmax + 2 * (maxTx + maxRx) * 4;
		stage = partial + 2 * cwarps * (maxTx + maxRx) * 4;
		stage = (stage + 127) & ~127u;
		total = stage + stages * capBytes;
	}
};

struct GroupSmem {
	uint64_t* full;
	uint64_t* empty;
	int* tileMax;              // [2]: largest transmit / receive delay of the tile (bits of a float >= 0)
	const unsigned char* zero; // 16 zero bytes
	GroupStage* meta;
	float4* rxinfo;            // [maxRx]: (x, y, apodization / storage scale, 0)
	float2* txinfo;            // [maxTx]: (x, y)
	float* minT;
	float* maxT;
	float* minR;
	float* maxR;
	float* partMin;            // [consumer warps][maxTx + maxRx]
	float* partMax;
	unsigned char* stageBuf;
	unsigned nst;
	unsigned capBytes;
	unsigned maxE;
};

__device__ __forceinline__ GroupSmem carve_group(unsigned char* smem, const GroupLayout& lay, unsigned maxTx,
		unsigned maxRx, unsigned cwarps, unsigned nst, unsigned capBytes)
{
	GroupSmem s;
	s.full = reinterpret_cast<uint64_t*>(smem + lay.bars);
	s.empty = s.full + nst;
	s.tileMax = reinterpret_cast<int*>(smem + lay.tileMax);
	s.zero = smem + lay.zero;
	s.meta = reinterpret_cast<GroupStage*>(smem + lay.meta);
	s.rxinfo = reinterpret_cast<float4*>(smem + lay.rxinfo);
	s.txinfo = reinterpret_cast<float2*>(smem + lay.txinfo);
	s.minT = reinterpret_cast<float*>(smem + lay.minmax);
	s.maxT = s.minT + maxTx;
	s.minR = s.maxT + maxTx;
	s.maxR = s.minR + maxRx;
	s.partMin = reinterpret_cast<float*>(smem + lay.partial);
	s.partMax = s.partMin + cwarps * (maxTx + maxRx);
	s.stageBuf = smem + lay.stage;
	s.nst = nst;
	s.capBytes = capBytes;
	s.maxE = maxTx + maxRx;
	return s;
}

__device__ __forceinline__ void init_group_barriers(const GroupSmem& sm, int cwarps)
{
	if (threadIdx.x < 4) reinterpret_cast<unsigned*>(const_cast<unsigned char*>(sm.zero))[threadIdx.x] = 0u;
	if (threadIdx.x == 0) {
		for (unsigned s = 0; s < sm.nst; ++s) {
			mbar_init(&sm.full[s], 1);
			mbar_init(&sm.empty[s], cwarps);
		}
		fence_barrier_init();
	}
	__syncthreads();
}

// ------------------------------------------------------------- producer
// Lane l sizes window (transmitter t0 + l / kGroup, receiver g * kGroup + l %
// kGroup); a prefix sum over the lanes packs as many whole units as fit into
// the stage; lane 0 arms the stage's barrier and every lane copies its window.
template<typename SP>
__device__ bool group_produce(const DasParams& p, const GroupSmem& sm, int& it, float margin)
{
	using T = typename SP::T;
	const int nst = static_cast<int>(sm.nst);
	const unsigned capBytes = sm.capBytes;
	const unsigned winCap = (capBytes / kGroup) & ~15u;  // a unit always fits in one stage
	const int lane = threadIdx.x & 31;
	const int u = lane / kGroup, j = lane % kGroup;
	const int L = static_cast<int>(p.L);
	const size_t txStride = static_cast<size_t>(p.numRx) * p.sigStride;
	const T* sig = reinterpret_cast<const T*>(p.sig);
	const unsigned numGroups = (p.numRx + kGroup - 1) / kGroup;
	const int itStart = it;
	int s = it % nst;
	unsigned phase = static_cast<unsigned>(it / nst) & 1u;
	bool ok = true;
	for (unsigned g = 0; g < numGroups && ok; ++g) {
		const unsigned r = g * kGroup + j;
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
			const unsigned t = t0 + u;
			int lo = 0, kind = kEmptyWindow;
			unsigned wb = 0;
			bool interior = false;   // the window needs no clamping to the A-scan
			if (t < p.numTx && r < p.numRx) {
				const float a = __fadd_rn(sm.minT[t], sm.minR[r]);
				const float b = __fadd_rn(sm.maxT[t], sm.maxR[r]);
				interior = floorf(a) - margin >= 0.0f && floorf(b) + 1.0f + margin <= static_cast<float>(L - 1);
				const float lof = fmaxf(floorf(a) - margin, 0.0f);
				const float hif = fminf(floorf(b) + 1.0f + margin, static_cast<float>(L - 1));
				if (lof <= static_cast<float>(L - 2) && hif >= 1.0f && hif >= lof) {
					lo = static_cast<int>(lof) & ~(SP::kAlign - 1);
					const unsigned cnt = static_cast<unsigned>(static_cast<int>(hif) - lo + 1);
					wb = (cnt * static_cast<unsigned>(sizeof(T)) + 15u) & ~15u;
					if (wb > winCap) {
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
			// Bytes through the end of this lane's unit; the units that fit
			// form a prefix (the first one always fits: winCap * kGroup <= cap).
			const unsigned unitEnd = __shfl_sync(0xffffffffu, incl, u * kGroup + kGroup - 1);
			const bool fits = t < p.numTx && unitEnd <= capBytes;
			const int n = __popc(__ballot_sync(0xffffffffu, fits && j == 0));
			const unsigned globalBits = __ballot_sync(0xffffffffu, kind == kGlobalWindow && u < n);
			const unsigned interiorBits = __ballot_sync(0xffffffffu, interior && kind == 0);
			const unsigned total = __shfl_sync(0xffffffffu, incl, n * kGroup - 1);
			const unsigned excl = incl - wb;
			GroupStage& m = sm.meta[s];
			if (u < n) {
				m.base[u][j] = (kind == 0) ? static_cast<int>(excl / sizeof(T)) - lo : 0;
				if (j == 0) {
					const unsigned inside = ((interiorBits >> (u * kGroup)) & 0xffu) == 0xffu ? kUnitInterior : 0u;
					m.unit[u] = make_int2(static_cast<int>(t), static_cast<int>(((globalBits >> (u * kGroup)) & 0xffu) | inside));
				}
			}
			if (lane == 0) {
				m.count = n;
				m.lastOfGroup = (t0 + n >= p.numTx) ? 1 : 0;
				m.anyGlobal = globalBits != 0u ? 1 : 0;
			}
			__threadfence_block();
			__syncwarp();
			// The test hook leaves this stage unarmed: its consumers' wait runs out.
			const bool skip = p.testSkipStage != 0u && it - itStart + 1 == static_cast<int>(p.testSkipStage);
			if (lane == 0 && !skip) mbar_arrive_expect_tx(&sm.full[s], total);
			__syncwarp();
			if (u < n && wb > 0 && !skip) {
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
		for (int q = from; q < it; ++q) {
			if (!mbar_wait_bounded(&sm.full[q % nst], (q / nst) & 1, wait_limit(p))) {
				atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
				ok = false;
			}
		}
	}
	return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

// ------------------------------------------------------------- consumers
// A consumer thread forms PY grid points of one column (PY = 1, or 2
// neighbouring rows): each unit's gathers for every point are independent, so
// a warp has PY times the loads in flight between two waits, and a tile of
// PY x the rows stages windows that are only a little longer.
//
// The group's gathers of one unit into `acc` (point k's accumulators of the
// group's receivers). FULL: every receiver of the group exists.
template<typename SP, bool Q, bool FULL, int PY>
__device__ __forceinline__ void group_gathers(const DasParams& p, const int2 un, const int* base,
		const typename SP::T* buf, const typename SP::T* zero, bool anyGlobal, unsigned g, unsigned nrg,
		const float (&txv)[PY], const float (&rxd)[PY][kGroup], unsigned lastIdx, const Fixed& fx,
		float2 (&acc)[PY][kGroup])
{
	using T = typename SP::T;
	if (FULL && (un.y & kUnitInterior)) {
		if constexpr (PY == 2 && !Q && SP::kAnalytic) {
			// Two points: the two points' delay splits and accumulations as
			// packed FP32x2 operations, each half rounded as the scalar form
			// (fl(tx + rx), the round-down split against 2^23, k = d -
			// floor(d) exactly, then fma(1 - k, s[i], acc) and fma(k, s[i + 1],
			// acc) per component on the samples widened to FP32): the same
			// bits, half the instructions.
			const float2 tx2 = make_float2(txv[0], txv[1]);
			const float2 big = make_float2(8388608.0f, 8388608.0f);
			const float2 nbig = make_float2(-8388608.0f, -8388608.0f);
			const float2 m1 = make_float2(-1.0f, -1.0f);
			const float2 one = make_float2(1.0f, 1.0f);
#pragma unroll
			for (int j = 0; j < kGroup; ++j) {
				const float2 d = __fadd2_rn(tx2, make_float2(rxd[0][j], rxd[1][j]));
				const float2 t0 = __fadd2_rd(d, big);
				const float2 k = __ffma2_rn(__fadd2_rn(t0, nbig), m1, d);
				const float2 w0 = __ffma2_rn(k, m1, one);
				const T* s0 = buf + (static_cast<int>(__float_as_uint(t0.x) - 0x4B000000u) + base[j]);
				const T* s1 = buf + (static_cast<int>(__float_as_uint(t0.y) - 0x4B000000u) + base[j]);
				const float2 a0 = SP::load(s0), c0 = SP::load(s0 + 1), a1 = SP::load(s1), c1 = SP::load(s1 + 1);
				acc[0][j] = __ffma2_rn(make_float2(k.x, k.x), c0, __ffma2_rn(make_float2(w0.x, w0.x), a0, acc[0][j]));
				acc[1][j] = __ffma2_rn(make_float2(k.y, k.y), c1, __ffma2_rn(make_float2(w0.y, w0.y), a1, acc[1][j]));
			}
			return;
		}
#pragma unroll
		for (int j = 0; j < kGroup; ++j) {
#pragma unroll
			for (int k = 0; k < PY; ++k) {
				float w;
				const int i = Delay<Q>::split(txv[k], rxd[k][j], w, fx);
				SP::accumulate(buf + (i + base[j]), w, acc[k][j]);
			}
		}
	} else if (!anyGlobal) {
#pragma unroll
		for (int j = 0; j < kGroup; ++j) {
			if (FULL || static_cast<unsigned>(j) < nrg) {
#pragma unroll
				for (int k = 0; k < PY; ++k) {
					gather_staged<SP, Q>(buf, base[j], txv[k], rxd[k][j], lastIdx, fx, zero, acc[k][j]);
				}
			}
		}
	} else {
		const T* sig = reinterpret_cast<const T*>(p.sig) + static_cast<size_t>(un.x) * p.numRx * p.sigStride;
#pragma unroll
		for (int j = 0; j < kGroup; ++j) {
			if (FULL || static_cast<unsigned>(j) < nrg) {
#pragma unroll
				for (int k = 0; k < PY; ++k) {
					if ((un.y >> j) & 1) {
						gather_global<SP, Q>(sig + static_cast<size_t>(g * kGroup + j) * p.sigStride, txv[k], rxd[k][j],
								lastIdx, fx, acc[k][j]);
					} else {
						gather_staged<SP, Q>(buf, base[j], txv[k], rxd[k][j], lastIdx, fx, zero, acc[k][j]);
					}
				}
			}
		}
	}
}

// One unit u of stage m with its transmitter's delays txv: the group's gathers.
template<typename SP, bool Q, bool FULL, int PY>
__device__ __forceinline__ void group_unit(const DasParams& p, const GroupStage& m, int u, const float (&txv)[PY],
		const typename SP::T* buf, const typename SP::T* zero, bool anyGlobal, unsigned g, unsigned nrg,
		const float (&rxd)[PY][kGroup], unsigned lastIdx, const Fixed& fx, float2 (&acc)[PY][kGroup])
{
	const int2 un = m.unit[u];
	const int4 b0 = *reinterpret_cast<const int4*>(&m.base[u][0]);
	const int4 b1 = *reinterpret_cast<const int4*>(&m.base[u][4]);
	const int base[kGroup] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
	group_gathers<SP, Q, FULL, PY>(p, un, base, buf, zero, anyGlobal, g, nrg, txv, rxd, lastIdx, fx, acc);
}

// The units of stage m (at least one), each unit's transmit delays computed
// one unit ahead so that their square roots overlap the previous unit's gathers.
template<typename SP, bool Q, bool FULL, int PY>
__device__ __forceinline__ void group_stage_units(const DasParams& p, const GroupSmem& sm, const GroupStage& m,
		int count, const typename SP::T* buf, const typename SP::T* zero, bool anyGlobal, unsigned g, unsigned nrg,
		const float (&px)[PY], const float (&py)[PY], const float (&pz)[PY], const float (&rxd)[PY][kGroup],
		unsigned lastIdx, const Fixed& fx, float2 (&acc)[PY][kGroup])
{
	float txNext[PY];
	{
		const float2 e = sm.txinfo[m.unit[0].x];
#pragma unroll
		for (int k = 0; k < PY; ++k) txNext[k] = Delay<Q>::tx(p, e, px[k], py[k], pz[k], fx);
	}
	for (int u = 0; u < count; ++u) {
		float txv[PY];
#pragma unroll
		for (int k = 0; k < PY; ++k) txv[k] = txNext[k];
		if (u + 1 < count) {
			const float2 e = sm.txinfo[m.unit[u + 1].x];
#pragma unroll
			for (int k = 0; k < PY; ++k) txNext[k] = Delay<Q>::tx(p, e, px[k], py[k], pz[k], fx);
		}
		group_unit<SP, Q, FULL, PY>(p, m, u, txv, buf, zero, anyGlobal, g, nrg, rxd, lastIdx, fx, acc);
	}
}

template<typename SP, int CF, bool Q, int PY>
__device__ bool group_consume(const DasParams& p, const GroupSmem& sm, int& it, const float (&px)[PY],
		const float (&py)[PY], const float (&pz)[PY], const bool (&active)[PY], const unsigned (&pix)[PY],
		const Fixed& fx)
{
	using T = typename SP::T;
	const int nst = static_cast<int>(sm.nst);
	const unsigned capBytes = sm.capBytes;
	const unsigned lastIdx = p.L - 2;
	const T* zero = reinterpret_cast<const T*>(sm.zero);
	const unsigned numGroups = (p.numRx + kGroup - 1) / kGroup;
	float2 total[PY];
	CFState<CF> cf[PY];
#pragma unroll
	for (int k = 0; k < PY; ++k) total[k] = make_float2(0.f, 0.f);
	int s = it % nst;
	unsigned phase = static_cast<unsigned>(it / nst) & 1u;
	for (unsigned g = 0; g < numGroups; ++g) {
		const unsigned nrg = min(static_cast<unsigned>(kGroup), p.numRx - g * kGroup);
		float rxd[PY][kGroup];
		float2 acc[PY][kGroup];  // point k, receiver g * kGroup + j: its terms in transmitter order
#pragma unroll
		for (int j = 0; j < kGroup; ++j) {
			const float4 e = (static_cast<unsigned>(j) < nrg) ? sm.rxinfo[g * kGroup + j] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
			for (int k = 0; k < PY; ++k) {
				rxd[k][j] = (static_cast<unsigned>(j) < nrg) ? Delay<Q>::rx(p, e, px[k], py[k], pz[k], fx) : 0.0f;
				acc[k][j] = make_float2(0.f, 0.f);
			}
		}
		bool last = false;
		while (!last) {
			if (!mbar_wait_bounded(&sm.full[s], phase, wait_limit(p))) {
				atomicOr(p.errWord, DEVERR_WAIT_TIMEOUT);
				return false;
			}
			const GroupStage& m = sm.meta[s];
			const T* buf = reinterpret_cast<const T*>(sm.stageBuf + static_cast<size_t>(s) * capBytes);
			const int4 head = *reinterpret_cast<const int4*>(&m.count);
			if (nrg == static_cast<unsigned>(kGroup)) {
				group_stage_units<SP, Q, true, PY>(p, sm, m, head.x, buf, zero, head.z != 0, g, nrg, px, py, pz, rxd,
						lastIdx, fx, acc);
			} else {
				group_stage_units<SP, Q, false, PY>(p, sm, m, head.x, buf, zero, head.z != 0, g, nrg, px, py, pz, rxd,
						lastIdx, fx, acc);
			}
			last = head.y != 0;
			__syncwarp();
			if ((threadIdx.x & 31) == 0) mbar_arrive(&sm.empty[s]);
			++it;
			if (++s == nst) {
				s = 0;
				phase ^= 1u;
			}
		}
#pragma unroll
		for (int j = 0; j < kGroup; ++j) {
			if (static_cast<unsigned>(j) < nrg) {
				const float w = sm.rxinfo[g * kGroup + j].z;
#pragma unroll
				for (int k = 0; k < PY; ++k) {
					const float2 rs = receiver_sum(acc[k][j], w);
					total[k].x += rs.x;
					total[k].y += rs.y;
					cf[k].add(rs);
				}
			}
		}
	}
#pragma unroll
	for (int k = 0; k < PY; ++k) {
		if (active[k]) {
			const float v = SP::kAnalytic ? magnitude(total[k]) : total[k].x;
			p.value[pix[k]] = v * p.valueCoef;
			p.factor[pix[k]] = cf[k].result(p.numRx, p, total[k]);
		}
	}
	return true;
}

// One tile (bx, by) of one frame: TCOLS columns x TROWS * PY rows, thread
// (warp w, lane l) on column bx * TCOLS + (w % CW) * 32 + l and rows
// by * TROWS * PY + (w / CW) * PY + k, k < PY; `it` is the block's running
// stage counter. SPLIT: the block is the single-frame kernel's
// GroupShape<NCW, PY>::kWarps warps and this is its only tile, so the
// register split may happen here (a batch block walks many tiles with NCW + 1
// warps and never splits: setmaxnreg needs whole warpgroups, and a repeated
// .inc would wait for registers no warp gives back).
template<int S, int CF, bool ANALYTIC, int TCOLS, int TROWS, int PY = 1, bool SPLIT = false>
__device__ bool group_tile(const DasParams& p, const GroupSmem& sm, unsigned bx, unsigned by, int& it)
{
	using SP = Sample<ANALYTIC, S>;
	constexpr int CW = TCOLS / 32;      // warps per tile row
	constexpr int NCW = TROWS * CW;     // consumer warps of the block
	// Thread rows with grid points: p.tileRows (at most TROWS; a single-frame
	// launch may use shorter tiles so that the tiles fill whole waves). The
	// consumer warps beyond them take part in the set-up barriers and the
	// register split, then leave.
	const int rowsA = min(static_cast<int>(p.tileRows), TROWS);
	const int ncwa = rowsA * CW;
	const int warp = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;
	const bool producer = warp >= NCW;   // the producer warp (NCW), and the exiting warps of a split block
	const bool idle = !producer && warp >= ncwa;
	const unsigned col = bx * TCOLS + (warp % CW) * 32 + lane;
	const unsigned row0 = by * (rowsA * PY) + (warp / CW) * PY;
	const unsigned nE = p.numTx + p.numRx;

	// Threads beyond the grid's edge take the nearest grid point of the tile.
	float px[PY], py[PY], pz[PY];
	bool active[PY];
	unsigned pix[PY];
#pragma unroll
	for (int k = 0; k < PY; ++k) {
		const unsigned row = row0 + k;
		active[k] = !producer && !idle && col < p.ncols && row < p.nrows;
		pix[k] = col * p.nrows + row;
		px[k] = py[k] = pz[k] = 0.f;
		if (!producer && !idle) {
			const unsigned q = min(col, p.ncols - 1) * p.nrows + min(row, p.nrows - 1);
			px[k] = p.grid[3 * q];
			py[k] = p.grid[3 * q + 1];
			pz[k] = p.grid[3 * q + 2];
		}
	}
	if (threadIdx.x == 0) {
		sm.tileMax[0] = 0;
		sm.tileMax[1] = 0;
	}
	for (unsigned r = threadIdx.x; r < p.numRx; r += blockDim.x) {
		sm.rxinfo[r] = make_float4(__ldg(&p.rxXY[2 * r]), __ldg(&p.rxXY[2 * r + 1]), __ldg(&p.apod[r]) * p.invScale, 0.f);
	}
	for (unsigned t = threadIdx.x; t < p.numTx; t += blockDim.x) {
		sm.txinfo[t] = make_float2(__ldg(&p.txXY[2 * t]), __ldg(&p.txXY[2 * t + 1]));
	}
	// Per-warp min/max of every element's FP32 delay over the tile.
	if (!producer && !idle) {
		for (unsigned e = 0; e < nE; ++e) {
			const bool isTx = e < p.numTx;
			const unsigned r = e - p.numTx;
			const float ex = isTx ? __ldg(&p.txXY[2 * e]) : __ldg(&p.rxXY[2 * r]);
			const float ey = isTx ? __ldg(&p.txXY[2 * e + 1]) : __ldg(&p.rxXY[2 * r + 1]);
			float mn = 0.f, mx = 0.f;
#pragma unroll
			for (int k = 0; k < PY; ++k) {
				const float d = __fmul_rn(distance3d_z0(ex, ey, px[k], py[k], pz[k]), p.invCT);
				const float v = isTx ? __fadd_rn(p.signalOffset, d) : d;
				mn = (k == 0) ? v : fminf(mn, v);
				mx = (k == 0) ? v : fmaxf(mx, v);
			}
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
		for (int w = 1; w < ncwa; ++w) {
			mn = fminf(mn, sm.partMin[w * sm.maxE + e]);
			mx = fmaxf(mx, sm.partMax[w * sm.maxE + e]);
		}
		if (e < p.numTx) { sm.minT[e] = mn; sm.maxT[e] = mx; topT = fmaxf(topT, mx); }
		else { sm.minR[e - p.numTx] = mn; sm.maxR[e - p.numTx] = mx; topR = fmaxf(topR, mx); }
	}
	if (topT > 0.f) atomicMax(&sm.tileMax[0], __float_as_int(topT));
	if (topR > 0.f) atomicMax(&sm.tileMax[1], __float_as_int(topR));
	__syncthreads();

	const float topTx = __int_as_float(sm.tileMax[0]), topRx = __int_as_float(sm.tileMax[1]);
	const bool q = p.delayMode == 2 || (p.delayMode == 0 && topTx + topRx > kDeepDelaySamples);
	const Fixed fx = fixed_format(fmaxf(fmaxf(topTx, topRx), fabsf(p.signalOffset)));
	using Shape = GroupShape<NCW, PY>;
	static_assert(!SPLIT || Shape::kSplit, "only the split block shape splits its registers");
	if constexpr (SPLIT) {
		// Warpgroup-uniform branches (warps 0-15: consumers; 16-19: producer group).
		if (producer) {
			regs_dec<Shape::kProducerRegs>();
			if (warp != NCW) return true;
		} else {
			regs_inc<Shape::kConsumerRegs>();
		}
	}
	if (producer) return group_produce<SP>(p, sm, it, q ? 2.0f : 0.0f);
	if (idle) return true;
	return q ? group_consume<SP, CF, true, PY>(p, sm, it, px, py, pz, active, pix, fx)
	         : group_consume<SP, CF, false, PY>(p, sm, it, px, py, pz, active, pix, fx);
}

// Resident blocks per SM the register allocation is held to, by consumer
// warps. One frame: 5 for 4 consumer warps (at most 81 registers a thread;
// measured fastest on the 64-element frames even though 32 KiB stages let
// only 3 blocks in). Batches (every coherence factor in one kernel, more live
// state): 3 for 4 and 2 for 8 consumer warps (fewer spills than at 5 and 3;
// measured faster on the mixed batch).
template<int NCW, int PY = 1> constexpr int group_min_blocks()
{
	return PY == 2 ? 1 : (NCW == 4 ? 5 : (NCW == 8 ? 3 : 1));
}
template<int NCW> constexpr int group_batch_min_blocks() { return NCW == 4 ? 3 : (NCW == 8 ? 2 : 1); }

template<int S, int CF, bool ANALYTIC, int TCOLS, int TROWS, int PY>
__global__ void __launch_bounds__(GroupShape<TROWS * TCOLS / 32, PY>::kWarps * 32,
		group_min_blocks<TROWS * TCOLS / 32, PY>())
das_group_kernel(DasParams p)
{
	constexpr int NCW = TROWS * TCOLS / 32;
	extern __shared__ __align__(128) unsigned char smem[];
	const GroupLayout lay(p.numTx, p.numRx, NCW, p.stageBytes, p.stages);
	const GroupSmem sm = carve_group(smem, lay, p.numTx, p.numRx, NCW, p.stages, p.stageBytes);
	init_group_barriers(sm, min(static_cast<int>(p.tileRows), TROWS) * (TCOLS / 32));   // consumer warps with grid points
	int it = 0;
	group_tile<S, CF, ANALYTIC, TCOLS, TROWS, PY, GroupShape<NCW, PY>::kSplit>(p, sm, blockIdx.x, blockIdx.y, it);
}

template<int S, int CF, bool ANALYTIC, int TCOLS, int TROWS, int PY = 1>
cudaError_t launch_group_one(const DasParams& p, cudaStream_t stream)
{
	constexpr int NCW = TROWS * TCOLS / 32;
	using Shape = GroupShape<NCW, PY>;
	const auto kernel = das_group_kernel<S, CF, ANALYTIC, TCOLS, TROWS, PY>;
	const GroupLayout lay(p.numTx, p.numRx, NCW, p.stageBytes, p.stages);
	cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lay.total));
	if (e != cudaSuccess) return e;
	if constexpr (Shape::kSplit) {
		// The register split assumes the launch allocation it was balanced
		// against; a build that allocates otherwise is not launched.
		cudaFuncAttributes fa{};
		if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
		if (fa.numRegs != Shape::kLaunchRegs) return cudaErrorInvalidConfiguration;
	}
	const unsigned tileH = min(p.tileRows, static_cast<unsigned>(TROWS)) * PY;
	const dim3 grid((p.ncols + TCOLS - 1) / TCOLS, (p.nrows + tileH - 1) / tileH);
	kernel<<<grid, Shape::kWarps * 32, lay.total, stream>>>(p);
	return cudaGetLastError();
}

// Tile shapes (columns x thread rows): 32 x 4, 32 x 8, 32 x 16, and 64 x 1-8
// (blocks of 4 or 8 thread rows); a thread row is one grid row, or two with
// two points per thread (p.pointsPerThread == 2: 64 x 2-16 grid rows).
template<int S, int CF, bool ANALYTIC>
cudaError_t launch_group_rows(const DasParams& p, cudaStream_t stream)
{
	if (p.tileCols == 64) {   // 1-8 thread rows: blocks of 4 or 8, the rest of the rows idle
		if (p.pointsPerThread == 2) {
			// (5-8 rows on the 20-warp block with the register split: 64 x 14
			// tiles there measured 1.437 ms against 1.481 ms on a 15-warp
			// block at 128 registers a thread)
			return p.tileRows <= 4 ? launch_group_one<S, CF, ANALYTIC, 64, 4, 2>(p, stream)
			                       : launch_group_one<S, CF, ANALYTIC, 64, 8, 2>(p, stream);
		}
		return p.tileRows <= 4 ? launch_group_one<S, CF, ANALYTIC, 64, 4>(p, stream)
		                       : launch_group_one<S, CF, ANALYTIC, 64, 8>(p, stream);
	}
	switch (p.tileRows) {
	case 4: return launch_group_one<S, CF, ANALYTIC, 32, 4>(p, stream);
	case 16: return launch_group_one<S, CF, ANALYTIC, 32, 16>(p, stream);
	default: return launch_group_one<S, CF, ANALYTIC, 32, 8>(p, stream);
	}
}

template<int S>
cudaError_t launch_group_cf(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	if (!analytic) {
		return (cf == CF_SCF) ? launch_group_rows<S, CF_SCF, false>(p, stream) : launch_group_rows<S, CF_NONE, false>(p, stream);
	}
	switch (cf) {
	case CF_PCF: return launch_group_rows<S, CF_PCF, true>(p, stream);
	case CF_SCF: return launch_group_rows<S, CF_SCF, true>(p, stream);
	case CF_MF: return launch_group_rows<S, CF_MF, true>(p, stream);
	default: return launch_group_rows<S, CF_NONE, true>(p, stream);
	}
}

template<int S, bool ANALYTIC, int TCOLS, int TROWS, int PY>
__device__ __forceinline__ bool group_tile_any_cf(const DasParams& p, int cf, const GroupSmem& sm, unsigned bx,
		unsigned by, int& it)
{
	if (!ANALYTIC) {
		return (cf == CF_SCF) ? group_tile<S, CF_SCF, false, TCOLS, TROWS, PY>(p, sm, bx, by, it)
		                      : group_tile<S, CF_NONE, false, TCOLS, TROWS, PY>(p, sm, bx, by, it);
	}
	switch (cf) {
	case CF_PCF: return group_tile<S, CF_PCF, true, TCOLS, TROWS, PY>(p, sm, bx, by, it);
	case CF_SCF: return group_tile<S, CF_SCF, true, TCOLS, TROWS, PY>(p, sm, bx, by, it);
	case CF_MF: return group_tile<S, CF_MF, true, TCOLS, TROWS, PY>(p, sm, bx, by, it);
	default: return group_tile<S, CF_NONE, true, TCOLS, TROWS, PY>(p, sm, bx, by, it);
	}
}

// Two points per thread: one block per SM (168 registers on 8 consumer warps).
template<int NCW, int PY> constexpr int group_batch_blocks()
{
	return PY == 2 ? 1 : group_batch_min_blocks<NCW>();
}

// Many frames: persistent blocks walk the tiles of every frame in the batch.
template<int S, bool ANALYTIC, int TCOLS, int TROWS, int PY>
__global__ void __launch_bounds__((TROWS * TCOLS / 32 + 1) * 32, group_batch_blocks<TROWS * TCOLS / 32, PY>())
das_group_batch_kernel(const BatchDasFrame* __restrict__ frames, const BatchHeader* __restrict__ hdr,
		unsigned maxTx, unsigned maxRx, unsigned capBytes, unsigned stages)
{
	constexpr int NCW = TROWS * TCOLS / 32;
	extern __shared__ __align__(128) unsigned char smem[];
	__shared__ DasParams sp;
	__shared__ int sAbort;
	const GroupLayout lay(maxTx, maxRx, NCW, capBytes, stages);
	const GroupSmem sm = carve_group(smem, lay, maxTx, maxRx, NCW, stages, capBytes);
	if (threadIdx.x == 0) sAbort = 0;
	init_group_barriers(sm, NCW);
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
		const bool ok = group_tile_any_cf<S, ANALYTIC, TCOLS, TROWS, PY>(sp, frames[f].cf, sm, local % tilesX,
				local / tilesX, it);
		if (!ok) sAbort = 1;
	}
}

template<int S, bool ANALYTIC, int TCOLS, int TROWS, int PY = 1>
cudaError_t launch_group_batch_one(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		cudaStream_t stream)
{
	constexpr int NCW = TROWS * TCOLS / 32;
	const GroupLayout lay(c.maxTx, c.maxRx, NCW, c.stageBytes, c.stages);
	const auto kernel = das_group_batch_kernel<S, ANALYTIC, TCOLS, TROWS, PY>;
	cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lay.total));
	if (e != cudaSuccess) return e;
	unsigned blocks = c.blocks;
	if (blocks == 0) {  // as many resident blocks as the SMs hold
		int perSM = 0, dev = 0, sms = 0;
		if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, (NCW + 1) * 32, lay.total)) != cudaSuccess) return e;
		if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
		if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
		blocks = static_cast<unsigned>(sms) * static_cast<unsigned>(perSM > 0 ? perSM : 1);
	}
	kernel<<<blocks, (NCW + 1) * 32, lay.total, stream>>>(frames, hdr, c.maxTx, c.maxRx, c.stageBytes, c.stages);
	return cudaGetLastError();
}

template<int S, bool ANALYTIC>
cudaError_t group_batch_rows(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		cudaStream_t stream)
{
	if (c.tileCols == 64) {
		if (c.pointsPerThread == 2) {
			// 64 x 8 (9 warps), 64 x 14 (15 warps) or 64 x 16 (17 warps) grid
			// points: up to 16 warps an SM keep 128 registers a thread; a 17th
			// puts five warps on one of the SM's four register-file partitions
			// (96 registers a thread, and the two-point consumers spill).
			switch (c.tileRows) {
			case 4: return launch_group_batch_one<S, ANALYTIC, 64, 4, 2>(frames, hdr, c, stream);
			case 7: return launch_group_batch_one<S, ANALYTIC, 64, 7, 2>(frames, hdr, c, stream);
			default: return launch_group_batch_one<S, ANALYTIC, 64, 8, 2>(frames, hdr, c, stream);
			}
		}
		return c.tileRows == 4 ? launch_group_batch_one<S, ANALYTIC, 64, 4>(frames, hdr, c, stream)
		                       : launch_group_batch_one<S, ANALYTIC, 64, 8>(frames, hdr, c, stream);
	}
	switch (c.tileRows) {
	case 4: return launch_group_batch_one<S, ANALYTIC, 32, 4>(frames, hdr, c, stream);
	case 16: return launch_group_batch_one<S, ANALYTIC, 32, 16>(frames, hdr, c, stream);
	default: return launch_group_batch_one<S, ANALYTIC, 32, 8>(frames, hdr, c, stream);
	}
}

}  // namespace

// The launchers of one storage type S (instantiated by one source file each).
template<int S>
cudaError_t launch_das_group_storage(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	return launch_group_cf<S>(p, cf, analytic, stream);
}

template<int S>
cudaError_t launch_das_group_batch_storage(const BatchDasFrame* frames, const BatchHeader* hdr,
		const BatchDasConfig& c, bool analytic, cudaStream_t stream)
{
	return analytic ? group_batch_rows<S, true>(frames, hdr, c, stream) : group_batch_rows<S, false>(frames, hdr, c, stream);
}

// Shared memory of a block; 64-column tiles of 1-8 thread rows run in blocks
// of 4 or 8 (the kernel's compile-time rows).
inline size_t group_layout_bytes(unsigned numTx, unsigned numRx, unsigned tileCols, unsigned tileRows, unsigned capBytes,
		unsigned stages)
{
	const unsigned blockRows = tileCols == 64 ? (tileRows <= 4 ? 4u : 8u) : tileRows;
	return GroupLayout(numTx, numRx, blockRows * (tileCols / 32), capBytes, stages).total;
}

}  // namespace usgb
