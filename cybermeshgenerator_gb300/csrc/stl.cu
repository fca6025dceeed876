// stl.cu — STL images into PLC arrays: binary records decoded on the device, ASCII
// parsed on host threads, coincident vertices merged on the device.
//
// Semantics of the reference reader (src/io/stl.cpp): binary when the image size is
// exactly 84 + 50 n (:163-168), the three float32 vertices of each 50-byte record
// widened to double (:96-110); otherwise ASCII (:112-129, include/cmg/io/detail.hpp:
// 22-60): lines split on '\n', '#' comments removed, blank lines skipped, tokens
// separated by whitespace or ',', "vertex"/"VERTEX" records with three numbers that
// strtod converts whole without range error. Vertices are merged on their exact
// coordinate triple (+0 and -0 equal), numbered in order of first occurrence, and a
// merged point keeps its first occurrence's coordinates (:26-65). A NaN coordinate is
// an error here (the reference's ordered map has no defined behaviour for it).
//
// Device merge, deterministic: every vertex probes an open-addressing table keyed by
// the position of some vertex with the same coordinates (compared through the vertex
// array, which never changes), and the slot keeps the smallest position that maps to
// it (atomicMin). A vertex is a first occurrence when that minimum is its own
// position; the exclusive scan of those flags in position order numbers the points
// exactly as the reference's first-occurrence order does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

constexpr int kEmpty = -1;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    // a 64-bit finaliser (xor-shift-multiply rounds): spreads every input bit
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ uint64_t key_hash(double x, double y, double z) {
    // +0.0 canonicalises -0 to +0 so that equal coordinates hash alike
    const uint64_t a = static_cast<uint64_t>(__double_as_longlong(x + 0.0));
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(y + 0.0));
    const uint64_t c = static_cast<uint64_t>(__double_as_longlong(z + 0.0));
    return mix64(a ^ mix64(b ^ mix64(c)));
}

// Binary records: the vertices of record t start at byte 50 t + 12 of `rec` (the
// image from byte 84 on), two-byte aligned; little-endian float32.
__global__ void k_stl_extract(const uint16_t* __restrict__ rec, int64_t n, double* __restrict__ v) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint16_t* r = rec + 25 * t + 6;  // (50 t + 12) / 2
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const uint32_t bits = static_cast<uint32_t>(r[2 * k]) | (static_cast<uint32_t>(r[2 * k + 1]) << 16);
        v[9 * t + k] = static_cast<double>(__uint_as_float(bits));
    }
}

__global__ void k_nan_check(const double* __restrict__ v, int64_t n, int* __restrict__ flag) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && v[i] != v[i]) atomicExch(flag, 1);
}

__global__ void k_weld_insert(const double* __restrict__ v, int64_t nv, int* __restrict__ tab,
                              int* __restrict__ slot, int* __restrict__ first, uint64_t mask,
                              int* __restrict__ fail) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    const double x = v[3 * p], y = v[3 * p + 1], z = v[3 * p + 2];
    uint64_t h = key_hash(x, y, z) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        int o = tab[h];
        if (o == kEmpty) {
            o = atomicCAS(&tab[h], kEmpty, static_cast<int>(p));
            if (o == kEmpty) o = static_cast<int>(p);
        }
        if (o == static_cast<int>(p) ||
            (v[3 * o] == x && v[3 * o + 1] == y && v[3 * o + 2] == z)) {
            slot[p] = static_cast<int>(h);
            atomicMin(&first[h], static_cast<int>(p));
            return;
        }
        h = (h + 1) & mask;
    }
    atomicExch(fail, 1);  // unreachable: the table holds at least twice the vertices
}

__global__ void k_weld_flags(int64_t nv, const int* __restrict__ slot, const int* __restrict__ first,
                             int* __restrict__ flag) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p < nv) flag[p] = first[slot[p]] == static_cast<int>(p) ? 1 : 0;
}

__global__ void k_weld_emit(int64_t nv, const double* __restrict__ v, const int* __restrict__ slot,
                            const int* __restrict__ first, const int64_t* __restrict__ rank,
                            double* __restrict__ pts, int* __restrict__ idx) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    const int f = first[slot[p]];
    const int64_t r = rank[f];
    idx[p] = static_cast<int>(r);
    if (f == static_cast<int>(p)) {
        pts[3 * r] = v[3 * p];
        pts[3 * r + 1] = v[3 * p + 1];
        pts[3 * r + 2] = v[3 * p + 2];
    }
}

struct StlWork {
    Arena arena;
    std::mutex mu;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float ms[3] = {0.f, 0.f, 0.f};  // last call: upload, decode + merge, download
};
StlWork& stl_work() {
    static StlWork w[64];
    int dev = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    return w[dev & 63];
}

bool is_space(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// strtod converting the whole token without ERANGE (std::stod's acceptance).
bool to_real(const char* s, size_t n, double& out) {
    char buf[128];
    std::string big;
    const char* z;
    if (n < sizeof(buf)) {
        std::memcpy(buf, s, n);
        buf[n] = '\0';
        z = buf;
    } else {
        big.assign(s, n);
        z = big.c_str();
    }
    errno = 0;
    char* end = nullptr;
    const double v = std::strtod(z, &end);
    if (end == z || errno == ERANGE || static_cast<size_t>(end - z) != n) return false;
    out = v;
    return true;
}

// Parses the lines of [b, e) (whole lines) into vertex coordinates; the first error
// of the range, if any, in `err`.
void parse_range(const char* b, const char* e, std::vector<double>& v, std::string& err) {
    const char* tok[4];
    size_t tlen[4];
    while (b < e) {
        const char* nl = static_cast<const char*>(std::memchr(b, '\n', static_cast<size_t>(e - b)));
        const char* le = nl ? nl : e;
        const char* hash = static_cast<const char*>(std::memchr(b, '#', static_cast<size_t>(le - b)));
        const char* end = hash ? hash : le;
        int nt = 0;
        const char* c = b;
        while (c < end) {
            while (c < end && (is_space(static_cast<unsigned char>(*c)) || *c == ',')) ++c;
            if (c >= end) break;
            const char* s = c;
            while (c < end && !is_space(static_cast<unsigned char>(*c)) && *c != ',') ++c;
            if (nt < 4) {
                tok[nt] = s;
                tlen[nt] = static_cast<size_t>(c - s);
            }
            ++nt;
        }
        b = nl ? nl + 1 : e;
        if (nt == 0) continue;
        const bool vert = (tlen[0] == 6 && (std::memcmp(tok[0], "vertex", 6) == 0 ||
                                            std::memcmp(tok[0], "VERTEX", 6) == 0));
        if (!vert) continue;
        if (nt < 4) {
            err = ".stl: short vertex record";
            return;
        }
        double x, y, z;
        if (!to_real(tok[1], tlen[1], x) || !to_real(tok[2], tlen[2], y) ||
            !to_real(tok[3], tlen[3], z)) {
            err = ".stl: non-numeric vertex coordinate";
            return;
        }
        v.push_back(x);
        v.push_back(y);
        v.push_back(z);
    }
}

// ASCII image -> flat vertex coordinates, on up to `threads` host threads over
// newline-aligned chunks; the first error in document order is reported.
void parse_ascii(const char* b, size_t len, std::vector<double>& v) {
    unsigned hw = std::thread::hardware_concurrency();
    size_t nchunk = len < (1u << 20) ? 1 : std::min<size_t>(hw ? hw : 1, 64);
    std::vector<const char*> cut(nchunk + 1);
    cut[0] = b;
    for (size_t i = 1; i < nchunk; ++i) {
        const char* p = b + len * i / nchunk;
        if (p < cut[i - 1]) p = cut[i - 1];
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(b + len - p)));
        cut[i] = nl ? nl + 1 : b + len;
    }
    cut[nchunk] = b + len;
    std::vector<std::vector<double>> part(nchunk);
    std::vector<std::string> err(nchunk);
    std::vector<std::thread> th;
    for (size_t i = 1; i < nchunk; ++i)
        th.emplace_back([&, i] { parse_range(cut[i], cut[i + 1], part[i], err[i]); });
    parse_range(cut[0], cut[1], part[0], err[0]);
    for (auto& t : th) t.join();
    for (size_t i = 0; i < nchunk; ++i) {
        if (!err[i].empty()) throw std::invalid_argument(err[i]);
        v.insert(v.end(), part[i].begin(), part[i].end());
    }
}

}  // namespace

void stl_read(const char* bytes, size_t len, HostVec<double>& pts, HostVec<int>& tris,
              cudaStream_t st) {
    bool binary = false;
    uint32_t n = 0;
    if (len >= 84) {
        std::memcpy(&n, bytes + 80, 4);
        binary = len == 84u + 50ull * n;
    }
    std::vector<double> hv;
    if (!binary) parse_ascii(bytes, len, hv);
    const int64_t nv = binary ? 3 * static_cast<int64_t>(n) : static_cast<int64_t>(hv.size() / 3);
    if (nv == 0 || nv % 3 != 0)
        throw std::invalid_argument(".stl: vertex count is not a positive multiple of 3");
    if (nv >= (int64_t(1) << 30)) throw std::invalid_argument(".stl: too many vertices");

    StlWork& W = stl_work();
    std::lock_guard<std::mutex> lk(W.mu);
    uint64_t S = 1;
    while (S < 2 * static_cast<uint64_t>(nv)) S <<= 1;
    Arena& A = W.arena;
    auto plan = [&](char** raw, double** v, int** tab, int** slot, int** first, int** flag,
                    int64_t** rank, int64_t** stmp, double** dp, int** di, int** fl) {
        A.reset();
        *raw = binary ? A.take<char>(50ull * n + 16) : nullptr;
        *v = A.take<double>(3 * nv);
        *tab = A.take<int>(S);
        *slot = A.take<int>(nv);
        *first = A.take<int>(S);
        *flag = A.take<int>(nv);
        *rank = A.take<int64_t>(nv + 1);
        *stmp = A.take<int64_t>(scan_tmp_elems(nv));
        *dp = A.take<double>(3 * nv);
        *di = A.take<int>(nv);
        *fl = A.take<int>(2);
    };
    char* raw;
    double *v, *dp;
    int *tab, *slot, *first, *flag, *di, *fl;
    int64_t *rank, *stmp;
    A.clear_need();
    plan(&raw, &v, &tab, &slot, &first, &flag, &rank, &stmp, &dp, &di, &fl);
    if (A.overflowed()) {
        A.reserve(A.need());
        plan(&raw, &v, &tab, &slot, &first, &flag, &rank, &stmp, &dp, &di, &fl);
    }
    if (!W.ev[0])
        for (cudaEvent_t& e : W.ev) CMG_CUDA(cudaEventCreate(&e));
    CMG_CUDA(cudaEventRecord(W.ev[0], st));
    if (binary) {
        CMG_CUDA(cudaMemcpyAsync(raw, bytes + 84, 50ull * n, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaEventRecord(W.ev[1], st));
        k_stl_extract<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(
            reinterpret_cast<const uint16_t*>(raw), n, v);
        CMG_LAUNCH();
    } else {
        CMG_CUDA(cudaMemcpyAsync(v, hv.data(), sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaEventRecord(W.ev[1], st));
    }
    CMG_CUDA(cudaMemsetAsync(fl, 0, 2 * sizeof(int), st));
    CMG_CUDA(cudaMemsetAsync(tab, 0xff, sizeof(int) * S, st));          // kEmpty
    CMG_CUDA(cudaMemsetAsync(first, 0x7f, sizeof(int) * S, st));        // > any position
    const unsigned g3 = static_cast<unsigned>((3 * nv + 255) / 256), gv = static_cast<unsigned>((nv + 255) / 256);
    k_nan_check<<<g3, 256, 0, st>>>(v, 3 * nv, fl);
    CMG_LAUNCH();
    k_weld_insert<<<gv, 256, 0, st>>>(v, nv, tab, slot, first, S - 1, fl + 1);
    CMG_LAUNCH();
    k_weld_flags<<<gv, 256, 0, st>>>(nv, slot, first, flag);
    CMG_LAUNCH();
    exclusive_scan(flag, rank, nv, stmp, st);
    k_weld_emit<<<gv, 256, 0, st>>>(nv, v, slot, first, rank, dp, di);
    CMG_LAUNCH();
    CMG_CUDA(cudaEventRecord(W.ev[2], st));
    int hf[2] = {0, 0};
    int64_t np = 0;
    CMG_CUDA(cudaMemcpyAsync(hf, fl, sizeof(hf), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaMemcpyAsync(&np, rank + nv, sizeof(np), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    if (hf[0]) throw std::invalid_argument(".stl: NaN vertex coordinate");
    if (hf[1]) throw std::runtime_error("stl: vertex table overflow");
    pts.resize(static_cast<size_t>(3 * np));
    tris.resize(static_cast<size_t>(nv));
    CMG_CUDA(cudaMemcpyAsync(pts.data(), dp, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaMemcpyAsync(tris.data(), di, sizeof(int) * nv, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaEventRecord(W.ev[3], st));
    CMG_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 3; ++k) CMG_CUDA(cudaEventElapsedTime(&W.ms[k], W.ev[k], W.ev[k + 1]));
}

void stl_last_timing(float* upload_ms, float* merge_ms, float* download_ms) {
    StlWork& W = stl_work();
    std::lock_guard<std::mutex> lk(W.mu);
    *upload_ms = W.ms[0];
    *merge_ms = W.ms[1];
    *download_ms = W.ms[2];
}

}  // namespace cmg::gpu
