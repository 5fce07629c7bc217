// Force-included ahead of the reference headers by oracle/build_ref.sh.
// CCCL 3 (CUDA 13) removed thrust::identity and cub::Min/cub::Sum, which the
// reference still names (running_stats.h:46, early_break.h:179-190); these
// restore them with the same meaning.  <random> is used by early_break.h:50
// without an include of its own.
#pragma once
#include <random>
#include <algorithm>
#include <cuda/functional>
#include <cuda/std/functional>
#include <thrust/functional.h>
namespace thrust {
template <typename T>
struct identity {
  __host__ __device__ const T& operator()(const T& x) const { return x; }
};
}  // namespace thrust
namespace cub {
using Min = ::cuda::minimum<>;
using Sum = ::cuda::std::plus<>;
}  // namespace cub
