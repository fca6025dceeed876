// cmg_util.h — host-side utilities shared by the engine translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace cmg::gpu {

// A CUDA call failed; carries the call site for the C ABI's error buffer.
struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess)
        throw CudaError(e, std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" +
                               std::to_string(line) + ")");
}
#define CMG_CUDA(x) ::cmg::gpu::cuda_check((x), #x, __FILE__, __LINE__)

// Every device allocation of the library goes through here. A test can make some of
// them fail on the host (set_alloc_failures, cmg_debug_fail_device_allocs): such an
// allocation returns cudaErrorMemoryAllocation without calling cudaMalloc.
cudaError_t device_alloc_raw(void** p, size_t bytes);
template <typename T>
inline cudaError_t device_alloc(T** p, size_t bytes) {
    return device_alloc_raw(reinterpret_cast<void**>(p), bytes);
}
// The next `skip` device allocations succeed, the `count` after them fail.
void set_alloc_failures(int skip, int count);
// Kernels launched by this library (process-wide), for launch accounting.
void note_launch(int n = 1);
long long launches();
#define CMG_LAUNCH()                                                                  \
    do {                                                                              \
        ::cmg::gpu::note_launch();                                                    \
        ::cmg::gpu::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__); \
    } while (0)

// exclusive prefix sum: out[i] = sum_{j<i} in[j] for i in [0, n], out[n] = total.
// tmp holds scan_tmp_elems(n) int64 values.
void exclusive_scan(const int* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t st);
void exclusive_scan(const int64_t* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t st);
size_t scan_tmp_elems(int64_t n);

// Stable LSD radix sort of (key, value) pairs on the low key_bits bits, in place.
size_t radix_sort_tmp_bytes(int64_t n);
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, int64_t n, int key_bits, void* tmp,
                      cudaStream_t st);

// Bump allocator over one device buffer. reset() before each pipeline; grows (by
// reallocating, outside any capture) when a pipeline asks for more than it holds.
class Arena {
public:
    Arena() = default;
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;
    ~Arena() { release(); }

    void reserve(size_t bytes) {
        if (bytes <= cap_) return;
        release();  // a failed allocation leaves the arena empty (and reusable)
        CMG_CUDA(device_alloc(&base_, bytes));
        cap_ = bytes;
    }
    void reset() { used_ = 0; }
    // Returns nullptr when the arena is too small; need() then reports the size.
    template <typename T>
    T* take(size_t count) {
        size_t bytes = (sizeof(T) * count + 255) & ~size_t(255);
        size_t at = used_;
        used_ += bytes;
        need_ = used_ > need_ ? used_ : need_;
        if (used_ > cap_) return nullptr;
        return reinterpret_cast<T*>(static_cast<char*>(base_) + at);
    }
    size_t need() const { return need_; }
    size_t capacity() const { return cap_; }
    bool overflowed() const { return used_ > cap_; }
    void clear_need() { need_ = 0; }
    void release() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
        cap_ = 0;
    }

private:
    void* base_ = nullptr;
    size_t cap_ = 0;
    size_t used_ = 0;
    size_t need_ = 0;
};

}  // namespace cmg::gpu
