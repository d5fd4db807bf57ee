// Minimal stand-in for tbb::blocked_range (TBB is not installed here).
#pragma once
#include <cstddef>
namespace tbb {
template<typename T>
class blocked_range {
public:
	blocked_range(T b, T e, std::size_t grain = 1) : b_(b), e_(e), grain_(grain) {}
	T begin() const { return b_; }
	T end() const { return e_; }
	std::size_t size() const { return static_cast<std::size_t>(e_ - b_); }
	bool empty() const { return !(b_ < e_); }
	std::size_t grainsize() const { return grain_; }
private:
	T b_, e_;
	std::size_t grain_;
};
}  // namespace tbb
