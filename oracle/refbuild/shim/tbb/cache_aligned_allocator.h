// Minimal stand-in for tbb::cache_aligned_allocator (alignment is not needed
// for the results).
#pragma once
#include <memory>
namespace tbb {
template<typename T>
class cache_aligned_allocator : public std::allocator<T> {
public:
	using value_type = T;
	template<typename U> struct rebind { using other = cache_aligned_allocator<U>; };
	cache_aligned_allocator() noexcept = default;
	template<typename U> cache_aligned_allocator(const cache_aligned_allocator<U>&) noexcept {}
};
template<typename T, typename U>
bool operator==(const cache_aligned_allocator<T>&, const cache_aligned_allocator<U>&) { return true; }
template<typename T, typename U>
bool operator!=(const cache_aligned_allocator<T>&, const cache_aligned_allocator<U>&) { return false; }
}  // namespace tbb
