// Host-side checks of the preparation plan (usgb_tables.h), no GPU: for
// A-scan lengths 1..N, the radix plan multiplies to M, every stage has a
// butterfly and a division constant, the wavefront model prefers the chosen
// plan to the even power-of-two split, and the Hilbert pair table visits every
// bin once, pairs k with M - k, puts k <= M/2 first and carries
// cos/sin(pi k / M).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "usgb_tables.h"

using namespace usgb;
using namespace usgb::host;

int main(int argc, char** argv)
{
	unsigned lo = 1, hi = 40000, step = 97;
	if (argc == 4) { lo = std::atoi(argv[1]); hi = std::atoi(argv[2]); step = std::atoi(argv[3]); }
	int bad = 0, sizes = 0;
	for (unsigned L = lo; L <= hi; L += step) {
		FFTTables t;
		if (!make_fft_tables(L, t)) continue;
		++sizes;
		const unsigned M = t.M;
		unsigned prod = 1;
		for (int r : t.radices) prod *= static_cast<unsigned>(r);
		if (prod != M) { std::printf("L %u: radices multiply to %u, not %u\n", L, prod, M); ++bad; continue; }
		if (t.divMagic.size() != t.radices.size()) { std::printf("L %u: division constants\n", L); ++bad; }
		std::vector<unsigned> perm(M), binAt(M);
		for (unsigned k = 0; k < M; ++k) {
			unsigned kk = k, pos = 0, span = M;
			for (int r : t.radices) { span /= static_cast<unsigned>(r); pos += (kk % r) * span; kk /= r; }
			perm[k] = pos;
			binAt[pos] = k;
		}
		std::vector<int> seen(M, 0);
		for (unsigned i = 0; i < t.hilb.size(); ++i) {
			unsigned code;
			std::memcpy(&code, &t.hilb[i].z, sizeof(code));
			if (code == kHilbertSkip) continue;
			if (code == i) {
				const unsigned k = binAt[i];
				if (!(k == 0 || 2 * k == M)) { std::printf("L %u: self pair at bin %u\n", L, k); ++bad; }
				++seen[i];
				continue;
			}
			const unsigned q = code & ~kHilbertSwap;
			const bool swap = (code & kHilbertSwap) != 0u;
			if (q <= i || q >= M) { std::printf("L %u: partner %u of %u\n", L, q, i); ++bad; continue; }
			const unsigned k1 = binAt[swap ? q : i], k2 = binAt[swap ? i : q];
			if (k1 + k2 != M || 2 * k1 > M) { std::printf("L %u: pair %u %u\n", L, k1, k2); ++bad; }
			const double a = 3.14159265358979323846 * k1 / M;
			if (std::fabs(std::cos(a) - t.hilb[i].x) > 1e-7 || std::fabs(std::sin(a) - t.hilb[i].y) > 1e-7) {
				std::printf("L %u: cos/sin of bin %u\n", L, k1);
				++bad;
			}
			++seen[q];
			++seen[i];
		}
		for (unsigned pos = 0; pos < M; ++pos) {
			if (seen[pos] != 1) { std::printf("L %u: position %u visited %d times\n", L, pos, seen[pos]); ++bad; break; }
		}
		if (bad > 20) break;
	}
	// The cf2d length: four passes, 16 * 8 * 9 * 15.
	FFTTables c;
	make_fft_tables(32768, c);
	const std::vector<int> want = {16, 8, 9, 15};
	if (c.M != 17280 || c.radices != want) { std::printf("cf2d plan differs\n"); ++bad; }
	if (fft_plan_wavefronts(c.M, c.radices) >= fft_plan_wavefronts(c.M, {8, 8, 6, 9, 5})) {
		std::printf("cf2d plan not cheaper than 8*8*6*9*5\n");
		++bad;
	}
	std::printf("sizes %d bad %d\n", sizes, bad);
	return bad == 0 ? 0 : 1;
}
