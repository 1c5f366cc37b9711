// Shared device helpers for libskidgpu (sm_103a).
//
// Distances reproduce the reference's float arithmetic exactly: no FMA
// (explicit __fmul_rn/__fadd_rn), ((dx*dx + dy*dy) + dz*dz), and periodic
// images formed as fl(x +/- L) before the subtraction (kd.h:122-214,
// smooth1.c:72-75,104-107).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define SKID_LEAF 32          // points per tree leaf = one warp
#define SKID_FULL 0xffffffffu

namespace skid {

// Device status word bits (latched; read by the host after a sync).
enum : unsigned {
    ST_TIMEOUT = 1u,     // a bounded wait ran out
    ST_OVERFLOW = 2u,    // a capacity was exceeded
    ST_BADSTATE = 4u,
};

__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ float d2of(float dx, float dy, float dz)
{
    return fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
}

// Query-frame component: the query's periodic image nearest the candidate,
// then fl(image - c).  Same rule as the oracle's img_dx.
__device__ __forceinline__ float img_dx(float q, float c, float L, float h)
{
    float d0 = fsub(q, c);
    if (d0 > h) return fsub(fsub(q, L), c);
    if (d0 < -h) return fsub(fadd(q, L), c);
    return d0;
}

// Per-lane, per-box image class of a query coordinate: all candidates c in
// [lo,hi] have q-c in [q-hi, q-lo].  Returns 0 (no shift for any), -1 (all
// need q-L), +1 (all need q+L) or 2 (mixed: decide per candidate).
__device__ __forceinline__ int img_class(float q, float lo, float hi, float h)
{
    float a = fsub(q, hi), b = fsub(q, lo);   // a <= b
    if (a >= -h && b <= h) return 0;
    if (a > h) return -1;
    if (b < -h) return 1;
    return 2;
}

// Lower bound of the float squared distance from q (any periodic image) to
// a box, with an absolute per-dimension slack covering the roundings of
// fl(fl(q+sL) - c); conservative for culling.
__device__ __forceinline__ float box_lb1(float q, float lo, float hi, float L, bool per)
{
    float d = fmaxf(fmaxf(lo - q, q - hi), 0.0f);
    if (per) {
        float qp = q + L, qm = q - L;
        d = fminf(d, fmaxf(fmaxf(lo - qp, qp - hi), 0.0f));
        d = fminf(d, fmaxf(fmaxf(lo - qm, qm - hi), 0.0f));
    }
    float slack = 4.8e-7f * (fabsf(q) + (per ? L : 0.0f) + fmaxf(fabsf(lo), fabsf(hi)));
    return fmaxf(d - slack, 0.0f);
}

__device__ __forceinline__ float box_lb(float3 q, float4 lo, float4 hi, float3 L, bool per)
{
    float dx = box_lb1(q.x, lo.x, hi.x, L.x, per);
    float dy = box_lb1(q.y, lo.y, hi.y, L.y, per);
    float dz = box_lb1(q.z, lo.z, hi.z, L.z, per);
    return (dx * dx + dy * dy + dz * dz) * (1.0f - 4e-6f);
}

// Lower bound of the float squared distance between any point of box a and
// any point of box b (periodic images included): box_lb taken over every
// point of a, with the slack of a's largest coordinate.
__device__ __forceinline__ float boxbox_lb1(float alo, float ahi, float blo, float bhi, float L,
                                            bool per)
{
    float d = fmaxf(fmaxf(blo - ahi, alo - bhi), 0.0f);
    if (per) {
        d = fminf(d, fmaxf(fmaxf(blo - (ahi + L), (alo + L) - bhi), 0.0f));
        d = fminf(d, fmaxf(fmaxf(blo - (ahi - L), (alo - L) - bhi), 0.0f));
    }
    float slack = 4.8e-7f * (fmaxf(fabsf(alo), fabsf(ahi)) + (per ? L : 0.0f) +
                             fmaxf(fabsf(blo), fabsf(bhi)));
    return fmaxf(d - slack, 0.0f);
}

__device__ __forceinline__ float boxbox_lb(float4 alo, float4 ahi, float4 blo, float4 bhi, float3 L,
                                           bool per)
{
    float dx = boxbox_lb1(alo.x, ahi.x, blo.x, bhi.x, L.x, per);
    float dy = boxbox_lb1(alo.y, ahi.y, blo.y, bhi.y, L.y, per);
    float dz = boxbox_lb1(alo.z, ahi.z, blo.z, bhi.z, L.z, per);
    return (dx * dx + dy * dy + dz * dz) * (1.0f - 4e-6f);
}

// Spread the low 21 bits of v to every third bit.
__device__ __forceinline__ uint64_t spread3(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// 3-D Hilbert index of B-bit integer coordinates (3B bits), after
// J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707 (2004):
// the axes are turned into the curve's transposed form (undo the excess
// work level by level, then Gray-encode), whose bits are interleaved with x
// highest at each level.  Consecutive indices are face-adjacent cells, so a
// run of consecutive points stays compact (a Morton run jumps across the
// box at every high-level boundary), and the index at B-1 bits of the
// halved coordinates is this index's top 3(B-1) bits.
template <int B>
__device__ __forceinline__ uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z)
{
#pragma unroll
    for (int b = B - 1; b > 0; --b) {
        const uint32_t Q = 1u << b, P = Q - 1u;
        x ^= (x & Q) ? P : 0u;
        if (y & Q) {
            x ^= P;
        } else {
            const uint32_t t = (x ^ y) & P;
            x ^= t;
            y ^= t;
        }
        if (z & Q) {
            x ^= P;
        } else {
            const uint32_t t = (x ^ z) & P;
            x ^= t;
            z ^= t;
        }
    }
    y ^= x;
    z ^= y;
    uint32_t t = 0;
#pragma unroll
    for (int b = B - 1; b > 0; --b) t ^= (z & (1u << b)) ? (1u << b) - 1u : 0u;
    x ^= t;
    y ^= t;
    z ^= t;
    return (spread3(x) << 2) | (spread3(y) << 1) | spread3(z);
}

// A point's cell on the 2^21 grid of the cubic frame (lo, inv).
__device__ __forceinline__ uint3 grid21(float3 p, float3 lo, float3 inv)
{
    const float fx = fminf(fmaxf((p.x - lo.x) * inv.x, 0.0f), 2097151.0f);
    const float fy = fminf(fmaxf((p.y - lo.y) * inv.y, 0.0f), 2097151.0f);
    const float fz = fminf(fmaxf((p.z - lo.z) * inv.z, 0.0f), 2097151.0f);
    return make_uint3((uint32_t)fx, (uint32_t)fy, (uint32_t)fz);
}

// The 63-bit Hilbert key of a point (21 levels).
__device__ __forceinline__ uint64_t hilbert63(float3 p, float3 lo, float3 inv)
{
    const uint3 q = grid21(p, lo, inv);
    return hilbert3<21>(q.x, q.y, q.z);
}

// The 63-bit Morton key of a point (bits of x, y, z interleaved).
__device__ __forceinline__ uint64_t morton63(float3 p, float3 lo, float3 inv)
{
    const uint3 q = grid21(p, lo, inv);
    return (spread3(q.x) << 2) | (spread3(q.y) << 1) | spread3(q.z);
}

// The top 32 bits of hilbert63, from the 11 coarsest levels alone.
__device__ __forceinline__ uint64_t hilbert_top32(float3 p, float3 lo, float3 inv)
{
    const uint3 q = grid21(p, lo, inv);
    return hilbert3<11>(q.x >> 10, q.y >> 10, q.z >> 10) >> 1;
}

// Sort keys on either curve: 63 bits, or the top 32.
__device__ __forceinline__ uint64_t curve63(float3 p, float3 lo, float3 inv, bool hil)
{
    return hil ? hilbert63(p, lo, inv) : morton63(p, lo, inv);
}
__device__ __forceinline__ uint64_t curve_top32(float3 p, float3 lo, float3 inv, bool hil)
{
    return hil ? hilbert_top32(p, lo, inv) : morton63(p, lo, inv) >> 31;
}

// Order-preserving float <-> uint for atomic min/max.
__device__ __forceinline__ unsigned f2ord(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ void set_status(unsigned *st, unsigned bit) { atomicOr(st, bit); }

// Implicit complete binary tree over leaves (root 1, children 2i and 2i+1,
// leaves at [nLeafP2, 2 nLeafP2)), the heap layout of kd.h:6-15.
__device__ __forceinline__ int next_node(int c)
{
    // SETNEXT (kd.h:11-15): the next node in depth-first order after the
    // subtree of c -- drop the trailing one bits, then step right.
    return (c >> (__ffs(~c) - 1)) + 1;
}

struct TreeView {
    int n;               // points
    int nLeaf;           // leaves holding points
    int leafBase;        // nLeafP2: node index of leaf 0
    const float4 *pos;   // sorted points (x, y, z, mass)
    const float4 *lo;    // node boxes [2*leafBase]; lo.w: max ball2 below
    const float4 *hi;    // hi.w: flags
};

}  // namespace skid
