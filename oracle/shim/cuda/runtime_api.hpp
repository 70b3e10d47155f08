// Host-only stand-in for the few cuda-api-wrappers names the reference's
// host-side headers use (include/hyset/containers.hpp:14-60, index.hpp:251-313,
// collection.hpp:54-71).  It lets oracle/ref_driver.cu compile the reference's
// own host::allpairs / host::ppjoin on a machine without a GPU.  Memory is plain
// host memory; kernel launches are never reached by the driver (it builds the
// inverted index on the CPU), so `launch` does nothing.  Written for this
// project: it reproduces API names only, no third-party code.
#pragma once
#include <cstddef>
#include <cstring>
#include <memory>
#include <thrust/sort.h>

namespace cuda {
namespace memory {
struct region_t {
    void* start;
    size_t size;
};
inline void copy(void* dst, const void* src, size_t bytes) { std::memcpy(dst, src, bytes); }
inline void zero(region_t r) { std::memset(r.start, 0, r.size); }
namespace device {
inline void set(void* p, int v, size_t bytes) { std::memset(p, v, bytes); }
inline void zero(void* p, size_t bytes) { std::memset(p, 0, bytes); }
}  // namespace device
namespace managed {
template <typename T>
using unique_ptr = std::unique_ptr<T>;
template <typename T>
typename std::enable_if<!std::is_array<T>::value, std::unique_ptr<T>>::type make_unique() {
    return std::unique_ptr<T>(new T());
}
template <typename T>
typename std::enable_if<std::is_array<T>::value, std::unique_ptr<T>>::type make_unique(size_t n) {
    return std::unique_ptr<T>(new typename std::remove_extent<T>::type[n]());
}
}  // namespace managed
}  // namespace memory

struct launch_configuration_t {
    launch_configuration_t(int, int, int = 0) {}
};
constexpr int no_shared_memory = 0;

template <typename K, typename... Args>
inline void launch(K, launch_configuration_t, Args&&...) {}

namespace device {
struct device_t {
    int get_attribute(int) const { return 1; }
};
namespace current {
inline device_t get() { return device_t(); }
}  // namespace current
}  // namespace device
}  // namespace cuda
