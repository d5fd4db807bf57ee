// Minimal stand-in for the TBB partitioner tags.
#pragma once
namespace tbb {
class simple_partitioner {};
class auto_partitioner {};
}  // namespace tbb
