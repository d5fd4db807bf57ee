// Minimal stand-in for tbb::parallel_for over std::thread. The range is cut
// into chunks of at least the grain size and the chunks are handed out to a
// fixed number of threads (USGB_REF_THREADS, default hardware_concurrency).
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <thread>
#include <vector>
#include "blocked_range.h"
#include "partitioner.h"
namespace tbb {
inline unsigned shim_num_threads()
{
	if (const char* s = std::getenv("USGB_REF_THREADS")) {
		const int n = std::atoi(s);
		if (n > 0) return static_cast<unsigned>(n);
	}
	const unsigned n = std::thread::hardware_concurrency();
	return n ? n : 1U;
}
template<typename T, typename Body>
void parallel_for(const blocked_range<T>& r, const Body& body)
{
	const std::size_t n = r.size();
	if (n == 0) return;
	const unsigned nt = std::min<std::size_t>(shim_num_threads(), n);
	if (nt <= 1) { body(r); return; }
	const std::size_t grain = std::max<std::size_t>(r.grainsize(), std::max<std::size_t>(1, n / (nt * 8)));
	std::atomic<std::size_t> next{0};
	std::vector<std::thread> pool;
	for (unsigned t = 0; t < nt; ++t) {
		pool.emplace_back([&]() {
			for (;;) {
				const std::size_t b = next.fetch_add(grain);
				if (b >= n) break;
				const std::size_t e = std::min(n, b + grain);
				body(blocked_range<T>(r.begin() + static_cast<T>(b), r.begin() + static_cast<T>(e), r.grainsize()));
			}
		});
	}
	for (auto& th : pool) th.join();
}
template<typename T, typename Body, typename Partitioner>
void parallel_for(const blocked_range<T>& r, const Body& body, const Partitioner&)
{
	parallel_for(r, body);
}
}  // namespace tbb
