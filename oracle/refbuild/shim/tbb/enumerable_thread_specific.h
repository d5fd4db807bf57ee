// Minimal stand-in for tbb::enumerable_thread_specific: one copy of the
// exemplar per calling thread, created on first use.
#pragma once
#include <map>
#include <memory>
#include <mutex>
#include <thread>
namespace tbb {
template<typename T>
class enumerable_thread_specific {
public:
	explicit enumerable_thread_specific(const T& exemplar) : exemplar_(exemplar) {}
	T& local()
	{
		std::lock_guard<std::mutex> lock(m_);
		auto& p = items_[std::this_thread::get_id()];
		if (!p) p = std::make_unique<T>(exemplar_);
		return *p;
	}
private:
	T exemplar_;
	std::mutex m_;
	std::map<std::thread::id, std::unique_ptr<T>> items_;
};
}  // namespace tbb
