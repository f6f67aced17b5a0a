// Device helpers shared by the BEM kernels: 3-vectors, the analytic
// triangle integrals, and bulk (TMA) global->shared staging with bounded
// mbarrier waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace omg {
namespace dev {

struct d3 {
    double x, y, z;
};
__device__ __forceinline__ d3 mk(double x, double y, double z) { return {x, y, z}; }
__device__ __forceinline__ d3 ld3(const double* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double norm(d3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Record layouts (doubles) -- must match the host-side constants.
// SREC: p0[0..2] p1[3..5] p2[6..8] n[9..11] area[12] len[13..15] en[16..24]
// PREC: p0..p2[0..8] n[9..11] area[12] D[13..21] U[22..30]
// QREC: q points [0..47] (x,y,z per point), area[48]

// Triangle::solid_angle (OpenMEEG/include/triangle.h:123-136)
__device__ __forceinline__ double solid_angle(d3 r0, d3 r1, d3 r2, double d0, double d1, double d2, d3 n,
                                              double area) {
    const double prod = d0 * d1 * d2;
    const double dd = 2 * area * dot(r0, n);
    return (fabs(dd) < 1e-10) ? 0.0 : 2 * atan2(dd, prod + (d0 * dot(r1, r2) + d1 * dot(r2, r0) + d2 * dot(r0, r1)));
}

// OperatorS::operator() (OpenMEEG/include/analytics.h:34-55): closed form of
// the integral over the record's triangle of 1/|y-x|.
__device__ __forceinline__ double operator_S(const double* s, d3 x) {
    const d3 r0 = ld3(s) - x, r1 = ld3(s + 3) - x, r2 = ld3(s + 6) - x;
    const double d0 = norm(r0), d1 = norm(r1), d2 = norm(r2);
    const d3 n = ld3(s + 9);
    double sum = dot(r0, ld3(s + 16)) * atanh(s[13] / (d0 + d1));
    sum += dot(r1, ld3(s + 19)) * atanh(s[14] / (d1 + d2));
    sum += dot(r2, ld3(s + 22)) * atanh(s[15] / (d2 + d0));
    return 2 * sum - dot(r0, n) * solid_angle(r0, r1, r2, d0, d1, d2, n, s[12]);
}

// P1SingleLayerPotential::operator() (OpenMEEG/include/analytics.h:87-119):
// the three P1-weighted double-layer integrals over the record's triangle.
__device__ __forceinline__ void p1_single_layer(const double* p, d3 x, double out[3]) {
    const d3 r0 = ld3(p) - x, r1 = ld3(p + 3) - x, r2 = ld3(p + 6) - x;
    const d3 n = ld3(p + 9);
    const double h = dot(r0, n);
    if (fabs(h) < 1e-10) {
        out[0] = out[1] = out[2] = 0.0;
        return;
    }
    const double area = p[12];
    const double d0 = norm(r0), d1 = norm(r1), d2 = norm(r2);
    const d3 D0 = ld3(p + 13), D1 = ld3(p + 16), D2 = ld3(p + 19);
    const d3 U0 = ld3(p + 22), U1 = ld3(p + 25), U2 = ld3(p + 28);
    const double l0 = log((d1 + dot(r1, U0)) / (d0 + dot(r0, U0)));
    const double l1 = log((d2 + dot(r2, U1)) / (d1 + dot(r1, U1)));
    const double l2 = log((d0 + dot(r0, U2)) / (d2 + dot(r2, U2)));
    const d3 S = U0 * l0 + U1 * l1 + U2 * l2;
    const double dd = 2 * h * area;
    const double den = d0 * d1 * d2 + (d0 * dot(r1, r2) + d1 * dot(r2, r0) + d2 * dot(r0, r1));
    const double omega = atan2(dd, den);
    const double inv = 1.0 / area;
    out[0] = (omega * dot(cross(r1, r2), n) + 0.5 * h * dot(D1, S)) * inv;
    out[1] = (omega * dot(cross(r2, r0), n) + 0.5 * h * dot(D2, S)) * inv;
    out[2] = (omega * dot(cross(r0, r1), n) + 0.5 * h * dot(D0, S)) * inv;
}

// operator_S and p1_single_layer of one triangle at one point (the S and P1
// records hold the same vertices, normal and area), with the vertex
// distances and the solid-angle arctangent computed once; each result is the
// expression of its own routine.
__device__ __forceinline__ double operator_S_p1(const double* s, const double* p, d3 x, double out[3]) {
    const d3 r0 = ld3(s) - x, r1 = ld3(s + 3) - x, r2 = ld3(s + 6) - x;
    const double d0 = norm(r0), d1 = norm(r1), d2 = norm(r2);
    const d3 n = ld3(s + 9);
    const double area = s[12];
    const double h = dot(r0, n);
    const double dd = 2 * area * h;   // = 2 h area exactly (doubling is exact)
    const double omega = atan2(dd, d0 * d1 * d2 + (d0 * dot(r1, r2) + d1 * dot(r2, r0) + d2 * dot(r0, r1)));
    double sum = dot(r0, ld3(s + 16)) * atanh(s[13] / (d0 + d1));
    sum += dot(r1, ld3(s + 19)) * atanh(s[14] / (d1 + d2));
    sum += dot(r2, ld3(s + 22)) * atanh(s[15] / (d2 + d0));
    const double S = 2 * sum - h * ((fabs(dd) < 1e-10) ? 0.0 : 2 * omega);
    if (fabs(h) < 1e-10) {
        out[0] = out[1] = out[2] = 0.0;
        return S;
    }
    const d3 D0 = ld3(p + 13), D1 = ld3(p + 16), D2 = ld3(p + 19);
    const d3 U0 = ld3(p + 22), U1 = ld3(p + 25), U2 = ld3(p + 28);
    const double l0 = log((d1 + dot(r1, U0)) / (d0 + dot(r0, U0)));
    const double l1 = log((d2 + dot(r2, U1)) / (d1 + dot(r1, U1)));
    const double l2 = log((d0 + dot(r0, U2)) / (d2 + dot(r2, U2)));
    const d3 L = U0 * l0 + U1 * l1 + U2 * l2;
    const double inv = 1.0 / area;
    out[0] = (omega * dot(cross(r1, r2), n) + 0.5 * h * dot(D1, L)) * inv;
    out[1] = (omega * dot(cross(r2, r0), n) + 0.5 * h * dot(D2, L)) * inv;
    out[2] = (omega * dot(cross(r0, r1), n) + 0.5 * h * dot(D0, L)) * inv;
    return S;
}

// ---------------------------------------------------------------------------
// Bulk copy (TMA engine, non-tensor form) into shared memory, completed on an
// mbarrier.  Waits are bounded: a wait that gives up reports OMG_ERR_TIMEOUT
// through `err` and the block skips its work.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// Returns true when the phase completed within the bound.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t max_iter = (1u << 20)) {
    for (uint32_t it = 0; it < max_iter; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Stage `nbytes` (multiple of 16, 16-byte aligned on both sides) of up to two
// contiguous global ranges into shared memory; all threads of the block must
// call it.  Returns false (for every thread) if the copy did not complete.
__device__ __forceinline__ bool stage_two(void* dstA, const void* srcA, uint32_t bytesA, void* dstB, const void* srcB,
                                          uint32_t bytesB, uint64_t* bar, int* err) {
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_expect_tx(bar, bytesA + bytesB);
        if (bytesA) bulk_g2s(dstA, srcA, bytesA, bar);
        if (bytesB) bulk_g2s(dstB, srcB, bytesB, bar);
    }
    __syncthreads();
    bool ok = mbar_wait_bounded(bar, 0);
    int any_fail = __syncthreads_or(!ok);
    if (any_fail) {
        if (threadIdx.x == 0) atomicExch(err, -8 /* OMG_ERR_TIMEOUT */);
        // the copies may still be landing in this block's shared memory: drain them (a much longer, still
        // bounded wait) before the block returns and its shared memory is reused
        mbar_wait_bounded(bar, 0, 1u << 28);
        __syncthreads();
        return false;
    }
    return true;
}

}  // namespace dev
}  // namespace omg
