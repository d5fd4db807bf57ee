// Host-side tables of the signal-preparation kernels, shared by every entry
// point: the polyphase FIR of the upsampler and the plan of the Hilbert FFT
// (radices, division constants, twiddles, digit-reversal permutation).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "usgb_internal.h"

namespace usgb {
namespace host {

constexpr double kPi = 3.14159265358979323846;

// FFTUtil::nextFastEvenSize (src/fft/FFTUtil.h:85-135): the smallest even
// n' >= n whose odd part has no prime factor above 5.
inline unsigned next_fast_even_size(unsigned n)
{
	if (n & 1U) ++n;
	for (;;) {
		unsigned m = n;
		while ((m & 1U) == 0) m >>= 1;
		while (m % 3 == 0) m /= 3;
		while (m % 5 == 0) m /= 5;
		if (m == 1) return n;
		n += 2;
	}
}

// Kaiser-windowed sinc of Interpolator::prepare (src/util/Interpolator.h:64-111,
// src/util/KaiserWindow.h:45-93), evaluated in float with the same mixed
// float/double expressions as Interpolator<float>.
inline std::vector<float> interpolator_taps(unsigned U, float halfTransitionWidth)
{
	const double kaiserTolerance = 1.0e-4;
	const float tol_dB = -20.0 * std::log10(kaiserTolerance);
	float beta;
	if (tol_dB > 50) {
		beta = 0.1102 * (tol_dB - 8.7);
	} else if (tol_dB > 21) {
		const double k = tol_dB - 21.0;
		beta = 0.5842 * std::pow(k, 0.4) + 0.07886 * k;
	} else {
		beta = 0.0;
	}
	const float finalTransitionWidth = (halfTransitionWidth * 2) / U;
	const double sz = std::ceil((tol_dB - 7.95) / (2.285 * finalTransitionWidth * kPi) + 1.0);
	const unsigned windowSize = static_cast<unsigned>(sz);
	const float twoUp = 2 * U;
	const unsigned n = static_cast<unsigned>(std::ceil((windowSize - 1) / twoUp) * twoUp) + 1U;

	std::vector<float> window(n);
	const float c1 = 2 / static_cast<float>(n - 1U);
	const float c2 = 1 / std::cyl_bessel_if(0.0f, beta);
	for (unsigned i = 0; i < n; ++i) {
		const float k = c1 * i - 1;
		float x = 1 - k * k;
		if (x < 0.0f) x = 0.0f;
		window[i] = c2 * std::cyl_bessel_if(0.0f, beta * std::sqrt(x));
	}
	const float numPeriods = (n - 1U) / twoUp;
	const double step = static_cast<double>(numPeriods - (-numPeriods)) / (n - 1U);
	std::vector<float> taps(n);
	for (unsigned i = 0; i < n; ++i) {
		const float xi = (i == 0) ? -numPeriods : static_cast<float>(-numPeriods + i * step);
		const double arg = kPi * xi;
		const double s = (std::abs(arg) < 1.0e-5) ? 1.0 - arg * arg / 6.0 : std::sin(arg) / arg;
		taps[i] = static_cast<float>(s);
		taps[i] *= window[i];
	}
	return taps;
}

// The fixed 4x FIR of the real-RF path, from the recipe stated in
// src/util/Interpolator4X.h:56-66 (kaiser(81, 5) .* sinc(linspace(-10, 10, 81))).
inline std::vector<float> interpolator4x_taps()
{
	const unsigned n = 80;
	const double beta = 5.0;
	const double i0b = std::cyl_bessel_i(0.0, beta);
	std::vector<float> h(n + 1);
	for (unsigned i = 0; i <= n; ++i) {
		const double r = 2.0 * i / n - 1.0;
		double arg = 1.0 - r * r;
		if (arg < 0.0) arg = 0.0;
		const double w = std::cyl_bessel_i(0.0, beta * std::sqrt(arg)) / i0b;
		const double xv = -10.0 + 20.0 * i / n;
		const double s = (xv == 0.0) ? 1.0 : std::sin(kPi * xv) / (kPi * xv);
		h[i] = static_cast<float>(s * w);
	}
	return h;
}

// The upsampler's FIR in polyphase form: poly[r][t] = h[r + tU] for the U
// phases, each padded to a multiple of 4 taps. Returns false when the FIR
// length is not 2UK + 1.
struct PolyTaps {
	std::vector<float> poly;
	unsigned tapsPerPhase = 1, tapsStride = 4;
};

inline bool make_poly_taps(bool analytic, unsigned U, PolyTaps& out)
{
	std::vector<float> taps;
	if (!analytic) {
		taps = interpolator4x_taps();
	} else if (U > 1) {
		taps = interpolator_taps(U, 0.2f);
	} else {
		taps = {1.0f};
	}
	const unsigned T = static_cast<unsigned>(taps.size());
	if (U > 1 && ((T - 1) % (2 * U) != 0)) return false;
	const unsigned K = (U > 1) ? (T - 1) / (2 * U) : 0;
	out.tapsPerPhase = 2 * K + 1;
	out.tapsStride = (out.tapsPerPhase + 3) & ~3u;
	out.poly.assign(static_cast<size_t>(U) * out.tapsStride, 0.f);
	for (unsigned r = 0; r < U; ++r) {
		for (unsigned t = 0; t < out.tapsPerPhase; ++t) {
			const unsigned j = r + t * U;
			out.poly[r * out.tapsStride + t] = (j < T) ? taps[j] : 0.f;
		}
	}
	return true;
}

// Weights of the input samples in the sum of the upsampled signal over
// [deadZone, L): y[bU + r] = sum_t poly[r][t] x[b + K - t] for b < ns, so
// x[j] enters that sum through every (t, r) whose output n = (j - K + t) U + r
// lies in [deadZone, L) with 0 <= j - K + t < ns (the DC mean of
// Util::removeDC, src/util/Util.h:1009-1018, as a dot product with the input).
inline std::vector<float> dc_coefficients(const PolyTaps& poly, unsigned U, unsigned ns, unsigned deadZone)
{
	const long long K = (poly.tapsPerPhase - 1) / 2;
	const long long L = static_cast<long long>(ns) * U;
	std::vector<float> c(ns);
	for (long long j = 0; j < static_cast<long long>(ns); ++j) {
		double sum = 0.0;
		for (long long t = 0; t < static_cast<long long>(poly.tapsPerPhase); ++t) {
			const long long b = j - K + t;
			if (b < 0 || b >= static_cast<long long>(ns)) continue;
			for (long long r = 0; r < static_cast<long long>(U); ++r) {
				const long long n = b * U + r;
				if (n >= static_cast<long long>(deadZone) && n < L) sum += poly.poly[r * poly.tapsStride + t];
			}
		}
		c[j] = static_cast<float>(sum);
	}
	return c;
}

// Copies the polyphase taps into the launch parameters (zero past them; the
// specialised FIR kernels read them only when they fit).
inline void set_param_taps(PrepParams& pp, const std::vector<float>& poly)
{
	std::fill(pp.paramTaps, pp.paramTaps + kParamTaps, 0.f);
	std::copy(poly.begin(), poly.begin() + std::min<size_t>(poly.size(), kParamTaps), pp.paramTaps);
}

// Plan of the Hilbert FFT of an L-sample A-scan: N = max(nextFastEvenSize(L +
// 1024), 2048) (src/util/HilbertEnvelope.h:152), computed as an M = N/2-point
// complex FFT.
struct FFTTables {
	unsigned N = 0, M = 0;
	std::vector<int> radices;                     // DIF order
	std::vector<unsigned long long> divMagic;     // per stage: ceil(2^40 / sub)
	std::vector<float2> tw;                       // two-level table (lo 128, then hi)
	unsigned twHiCount = 0;
	// Hilbert pass in digit-reversed position order (kHilbertSkip / the pair
	// encoding of PrepParams::hilb): entry p < hilb.size() is
	// (cos, sin)(pi k_lo / M), the partner's position and which of the two
	// positions holds k_lo, for the pair (k, M - k) whose lower position is p.
	std::vector<float4> hilb;
	// Stage tables: for stage s >= 1 (span Ms, radix R), W_Ms^j for j < Ms / R,
	// at stageTwOffset[s] (stage 0 reads the two-level table).
	std::vector<float2> stageTw;
	std::vector<unsigned> stageTwOffset;
};

// Shared-memory wavefronts of the in-place stages of `plan` over M points,
// one direction: each warp request (32 consecutive butterflies b of a stage,
// one of its R float2 loads or stores) costs the largest number of distinct
// 4-byte words any of the 32 banks holds.
inline double fft_plan_wavefronts(unsigned M, const std::vector<int>& plan)
{
	double total = 0.0;
	unsigned Ms = M;
	for (int R : plan) {
		const unsigned r = static_cast<unsigned>(R);
		const unsigned sub = Ms / r;
		const unsigned nb = M / r;
		for (unsigned w0 = 0; w0 < nb; w0 += 32) {
			const unsigned n = std::min(32u, nb - w0);
			for (unsigned q = 0; q < r; ++q) {
				unsigned words[64];
				for (unsigned l = 0; l < n; ++l) {
					const unsigned b = w0 + l;
					const unsigned blk = b / sub;
					const unsigned pos = blk * Ms + (b - blk * sub) + q * sub;
					words[2 * l] = 2 * pos;
					words[2 * l + 1] = 2 * pos + 1;
				}
				std::sort(words, words + 2 * n);
				const unsigned* end = std::unique(words, words + 2 * n);
				unsigned banks[32] = {};
				unsigned worst = 0;
				for (const unsigned* w = words; w != end; ++w) worst = std::max(worst, ++banks[*w % 32]);
				total += 2.0 * worst;   // the load and the store
			}
		}
		Ms = sub;
	}
	return total;
}

inline bool make_fft_tables(unsigned L, FFTTables& t)
{
	t.N = std::max(next_fast_even_size(L + 1024U), 2048U);
	t.M = t.N / 2;
	const unsigned M = t.M;
	unsigned m = M;
	int e2 = 0, e3 = 0, e5 = 0;
	while (m % 2 == 0) { m /= 2; ++e2; }
	while (m % 3 == 0) { m /= 3; ++e3; }
	while (m % 5 == 0) { m /= 5; ++e5; }
	if (m != 1) return false;
	// Few passes over the buffer (each pass reads and writes every point in
	// shared memory), without bank conflicts where possible. The odd part:
	// radix 15 for each 3 * 5 pair, radix 9 for the remaining 3^2, then a 3,
	// and 5; a single 2 pairs with a leftover 3 as radix 6. The power of two:
	// every non-increasing sequence of radices 16 / 8 / 4 / 2 with at most
	// one pass more than the fewest, each plan scored by the shared-memory
	// wavefronts of its passes (fft_plan_wavefronts); the power-of-two
	// radices run first (long blocks), the odd ones last, where the blocks are
	// short and odd strides keep the banks apart (cf2d, M = 17280:
	// 16 * 8 * 9 * 15, four passes; the first form took eight).
	std::vector<int> odd;
	int n15 = std::min(e3, e5);
	int r3 = e3 - n15, r5 = e5 - n15;
	bool two = e2 == 1;
	if (two && r3 % 2 == 1) { odd.push_back(6); two = false; --r3; }
	if (two) odd.push_back(2);
	for (int i = 0; i < r3 / 2; ++i) odd.push_back(9);
	if (r3 % 2 == 1) odd.push_back(3);
	for (int i = 0; i < r5; ++i) odd.push_back(5);
	for (int i = 0; i < n15; ++i) odd.push_back(15);
	std::vector<std::vector<int>> pow2;
	if (e2 > 1) {
		const int fewest = (e2 + 3) / 4;
		std::vector<int> cur;
		// Non-increasing sequences of 2^b (b = 4 .. 1) summing to e2 bits.
		auto rec = [&](auto&& self, int left, int maxBits) -> void {
			if (left == 0) { pow2.push_back(cur); return; }
			if (static_cast<int>(cur.size()) >= fewest + 1) return;
			for (int bits = std::min(maxBits, left); bits >= 1; --bits) {
				cur.push_back(1 << bits);
				self(self, left - bits, bits);
				cur.pop_back();
			}
		};
		rec(rec, e2, 4);
	} else {
		pow2.push_back({});
	}
	double best = 0.0;
	for (const auto& p2 : pow2) {
		std::vector<int> plan = p2;
		plan.insert(plan.end(), odd.begin(), odd.end());
		const double cost = fft_plan_wavefronts(M, plan);
		if (t.radices.empty() || cost < best || (cost == best && plan.size() < t.radices.size())) {
			best = cost;
			t.radices = plan;
		}
	}
	if (t.radices.size() > static_cast<size_t>(kMaxFFTStages)) return false;

	auto unit = [](double a) { return make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a))); };
	const unsigned S = kTwiddleSplit;
	t.twHiCount = (M + S - 1) / S;
	t.tw.resize(S + t.twHiCount);
	for (unsigned j = 0; j < S; ++j) t.tw[j] = unit(-2.0 * kPi * static_cast<double>(j) / M);
	for (unsigned q = 0; q < t.twHiCount; ++q) t.tw[S + q] = unit(-2.0 * kPi * static_cast<double>(q) * S / M);

	// Multiply-shift division by each stage's sub-block length:
	// floor(b / sub) = (b * ceil(2^40 / sub)) >> 40, exact for b, sub < 2^20.
	t.divMagic.clear();
	t.stageTw.clear();
	t.stageTwOffset.assign(t.radices.size(), 0);
	unsigned Ms = M;
	for (size_t s = 0; s < t.radices.size(); ++s) {
		const unsigned sub = Ms / static_cast<unsigned>(t.radices[s]);
		t.divMagic.push_back(((1ULL << 40) + sub - 1) / sub);
		if (s > 0) {
			t.stageTwOffset[s] = static_cast<unsigned>(t.stageTw.size());
			for (unsigned j = 0; j < sub; ++j) t.stageTw.push_back(unit(-2.0 * kPi * static_cast<double>(j) / Ms));
		}
		Ms = sub;
	}
	// Digit-reversed position of bin k after the in-place DIF stages:
	// k = k0 + r0 (k1 + r1 (k2 + ...)) sits at sum_s k_s * M / (r0 ... r_s).
	std::vector<unsigned> perm(M), binAt(M);
	for (unsigned k = 0; k < M; ++k) {
		unsigned kk = k, pos = 0, span = M;
		for (int r : t.radices) {
			span /= static_cast<unsigned>(r);
			pos += (kk % r) * span;
			kk /= r;
		}
		perm[k] = pos;
		binAt[pos] = k;
	}
	// Pairs (k, M - k) visited in position order: consecutive lanes then read
	// consecutive positions, and the partners' positions run consecutively
	// too (in k order, consecutive bins sit M / r0 apart: every lane on one
	// shared-memory bank). Each pair is handled from its lower position; the
	// last such position bounds the table.
	unsigned count = 0;
	for (unsigned pos = 0; pos < M; ++pos) {
		const unsigned q = perm[(M - binAt[pos]) % M];
		if (q >= pos) count = pos + 1;
	}
	t.hilb.assign(count, make_float4(0.f, 0.f, 0.f, 0.f));
	for (unsigned pos = 0; pos < count; ++pos) {
		const unsigned k = binAt[pos];
		const unsigned kp = (M - k) % M;
		const unsigned q = perm[kp];
		unsigned code = kHilbertSkip;
		float2 cs = make_float2(0.f, 0.f);
		if (q == pos) {
			code = pos;                        // k = 0 or k = M / 2
		} else if (q > pos) {
			const unsigned klo = std::min(k, kp);
			code = q | ((k == klo) ? 0u : kHilbertSwap);
			cs = unit(kPi * static_cast<double>(klo) / M);
		}
		float codeBits;
		std::memcpy(&codeBits, &code, sizeof(code));
		t.hilb[pos] = make_float4(cs.x, cs.y, codeBits, 0.f);
	}
	return true;
}

// Fills the FFT fields of `pp` from `t` (device table pointers set by the caller).
inline void set_fft_params(PrepParams& pp, const FFTTables& t)
{
	pp.M = t.M;
	pp.numStages = static_cast<int>(t.radices.size());
	for (size_t i = 0; i < t.radices.size(); ++i) {
		pp.radix[i] = t.radices[i];
		pp.divMagic[i] = t.divMagic[i];
		pp.stwOffset[i] = t.stageTwOffset[i];
	}
	pp.twHiCount = t.twHiCount;
	pp.hilbCount = static_cast<unsigned>(t.hilb.size());
	pp.stwCount = static_cast<unsigned>(t.stageTw.size());
}

}  // namespace host
}  // namespace usgb
