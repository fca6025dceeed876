// cmg_device.cuh — device arithmetic shared by the voxelization kernels.
//
// Reference-order FP64: every operation whose rounding must equal the reference
// CPU build (x86-64 SSE2, no fused multiply-add) is written with an explicit
// round-to-nearest intrinsic, so no compiler flag can contract or reorder it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cmg::gpu {

// ---------------------------------------------------------------- FP64, exact order
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

struct d3 {
    double x, y, z;
};

__device__ __forceinline__ d3 ld3(const double* p) { return {p[0], p[1], p[2]}; }

// Cell-centre coordinate corner + (i + 0.5) * h (voxelize.cpp:180-181, :187).
__device__ __forceinline__ double cell_center(double corner, int i, double h) {
    return dadd(corner, dmul(dadd(static_cast<double>(i), 0.5), h));
}

// floor((x - corner) / h) clamped to [0, n) (voxelize.cpp:82-89, :256-259).
__device__ __forceinline__ int cell_clamped(double x, double corner, double h, int n) {
    double f = floor(ddiv(dsub(x, corner), h));
    int i;
    if (f < 0.0) i = 0;                      // also covers -inf
    else if (f >= static_cast<double>(n)) i = n - 1;
    else i = static_cast<int>(f);
    return i;                                 // NaN lands in the last branch
}

// Rounded orient3d determinant in Shewchuk's operation order
// (src/predicates/predicates.cpp:2201-2222); optionally the permanent (:2237-2239).
__device__ __forceinline__ double o3d_fast(const d3& a, const d3& b, const d3& c,
                                           const d3& d, double* permanent) {
    double adx = dsub(a.x, d.x), ady = dsub(a.y, d.y), adz = dsub(a.z, d.z);
    double bdx = dsub(b.x, d.x), bdy = dsub(b.y, d.y), bdz = dsub(b.z, d.z);
    double cdx = dsub(c.x, d.x), cdy = dsub(c.y, d.y), cdz = dsub(c.z, d.z);
    double bdxcdy = dmul(bdx, cdy), cdxbdy = dmul(cdx, bdy);
    double cdxady = dmul(cdx, ady), adxcdy = dmul(adx, cdy);
    double adxbdy = dmul(adx, bdy), bdxady = dmul(bdx, ady);
    double det = dadd(dadd(dmul(adz, dsub(bdxcdy, cdxbdy)), dmul(bdz, dsub(cdxady, adxcdy))),
                      dmul(cdz, dsub(adxbdy, bdxady)));
    if (permanent)
        *permanent = dadd(dadd(dmul(dadd(fabs(bdxcdy), fabs(cdxbdy)), fabs(adz)),
                               dmul(dadd(fabs(cdxady), fabs(adxcdy)), fabs(bdz))),
                          dmul(dadd(fabs(adxbdy), fabs(bdxady)), fabs(cdz)));
    return det;
}

// Error-bound constants of the exact-arithmetic filter (predicates.cpp:617, :623),
// epsilon = 2^-53.
constexpr double kEps53 = 1.1102230246251565e-16;
constexpr double kO3dErrA = (7.0 + 56.0 * kEps53) * kEps53;
constexpr double kIspErrA = (16.0 + 224.0 * kEps53) * kEps53;

// Rounded insphere determinant in the reference's order (predicates.cpp:4050-4110).
__device__ __forceinline__ double isp_fast(const d3& a, const d3& b, const d3& c,
                                           const d3& d, const d3& e, double* permanent) {
    double aex = dsub(a.x, e.x), bex = dsub(b.x, e.x), cex = dsub(c.x, e.x), dex = dsub(d.x, e.x);
    double aey = dsub(a.y, e.y), bey = dsub(b.y, e.y), cey = dsub(c.y, e.y), dey = dsub(d.y, e.y);
    double aez = dsub(a.z, e.z), bez = dsub(b.z, e.z), cez = dsub(c.z, e.z), dez = dsub(d.z, e.z);
    double aexbey = dmul(aex, bey), bexaey = dmul(bex, aey), ab = dsub(aexbey, bexaey);
    double bexcey = dmul(bex, cey), cexbey = dmul(cex, bey), bc = dsub(bexcey, cexbey);
    double cexdey = dmul(cex, dey), dexcey = dmul(dex, cey), cd = dsub(cexdey, dexcey);
    double dexaey = dmul(dex, aey), aexdey = dmul(aex, dey), da = dsub(dexaey, aexdey);
    double aexcey = dmul(aex, cey), cexaey = dmul(cex, aey), ac = dsub(aexcey, cexaey);
    double bexdey = dmul(bex, dey), dexbey = dmul(dex, bey), bd = dsub(bexdey, dexbey);
    double abc = dadd(dsub(dmul(aez, bc), dmul(bez, ac)), dmul(cez, ab));
    double bcd = dadd(dsub(dmul(bez, cd), dmul(cez, bd)), dmul(dez, bc));
    double cda = dadd(dadd(dmul(cez, da), dmul(dez, ac)), dmul(aez, cd));
    double dab = dadd(dadd(dmul(dez, ab), dmul(aez, bd)), dmul(bez, da));
    double alift = dadd(dadd(dmul(aex, aex), dmul(aey, aey)), dmul(aez, aez));
    double blift = dadd(dadd(dmul(bex, bex), dmul(bey, bey)), dmul(bez, bez));
    double clift = dadd(dadd(dmul(cex, cex), dmul(cey, cey)), dmul(cez, cez));
    double dlift = dadd(dadd(dmul(dex, dex), dmul(dey, dey)), dmul(dez, dez));
    double det = dadd(dsub(dmul(dlift, abc), dmul(clift, dab)),
                      dsub(dmul(blift, cda), dmul(alift, bcd)));
    if (permanent) {
        double aezp = fabs(aez), bezp = fabs(bez), cezp = fabs(cez), dezp = fabs(dez);
        double p_ab = dadd(fabs(aexbey), fabs(bexaey)), p_bc = dadd(fabs(bexcey), fabs(cexbey));
        double p_cd = dadd(fabs(cexdey), fabs(dexcey)), p_da = dadd(fabs(dexaey), fabs(aexdey));
        double p_ac = dadd(fabs(aexcey), fabs(cexaey)), p_bd = dadd(fabs(bexdey), fabs(dexbey));
        double t1 = dmul(dadd(dadd(dmul(p_cd, bezp), dmul(p_bd, cezp)), dmul(p_bc, dezp)), alift);
        double t2 = dmul(dadd(dadd(dmul(p_da, cezp), dmul(p_ac, dezp)), dmul(p_cd, aezp)), blift);
        double t3 = dmul(dadd(dadd(dmul(p_ab, dezp), dmul(p_bd, aezp)), dmul(p_da, bezp)), clift);
        double t4 = dmul(dadd(dadd(dmul(p_bc, aezp), dmul(p_ac, bezp)), dmul(p_ab, cezp)), dlift);
        *permanent = dadd(dadd(dadd(t1, t2), t3), t4);
    }
    return det;
}

__device__ __forceinline__ int sgn(double v) { return v > 0.0 ? 1 : (v < 0.0 ? -1 : 0); }

// ---------------------------------------------------------------- warp helpers
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace cmg::gpu
