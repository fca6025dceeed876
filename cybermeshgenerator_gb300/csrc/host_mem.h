// host_mem.h — host memory for arrays that devices fill or read: a pool of reused
// page-locked blocks and an allocator that draws large arrays from it.
#pragma once

#include <cstddef>
#include <new>
#include <utility>
#include <vector>

namespace cmg::gpu {

// Page-locked host blocks, kept for reuse after release: a device-to-host copy
// into one runs at the link's rate (no staging through the driver's bounce
// buffers), and pinning is paid once per block rather than once per call. A block
// of `bytes` or more is returned with its capacity; when pinning fails the block is
// ordinary heap memory (*pinned = false). Released blocks beyond the pool's cap of
// cached bytes are freed. Thread-safe.
void* host_block_acquire(size_t bytes, size_t* cap, bool* pinned);
void host_block_release(void* p, size_t cap, bool pinned);

// Host allocation by size: 1 MiB and more from the page-locked block pool, less
// from the heap. host_large_free takes the size that was asked for.
void* host_large_alloc(size_t bytes);
void host_large_free(void* p, size_t bytes) noexcept;

// Allocator of large host arrays (PLC storage, device results): page-locked pool
// blocks above 1 MiB, and elements default-initialised, so that a resize does not
// write what a device copy is about to fill.
template <typename T>
struct HostAlloc {
    using value_type = T;
    HostAlloc() noexcept = default;
    template <typename U>
    HostAlloc(const HostAlloc<U>&) noexcept {}
    T* allocate(size_t n) { return static_cast<T*>(host_large_alloc(n * sizeof(T))); }
    void deallocate(T* p, size_t n) noexcept { host_large_free(p, n * sizeof(T)); }
    template <typename U>
    void construct(U* p) noexcept {
        ::new (static_cast<void*>(p)) U;
    }
    template <typename U, typename... A>
    void construct(U* p, A&&... a) {
        ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
    }
    template <typename U>
    bool operator==(const HostAlloc<U>&) const noexcept { return true; }
    template <typename U>
    bool operator!=(const HostAlloc<U>&) const noexcept { return false; }
};
template <typename T>
using HostVec = std::vector<T, HostAlloc<T>>;

}  // namespace cmg::gpu
