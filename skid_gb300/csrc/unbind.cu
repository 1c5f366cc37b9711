// Gravitational unbinding of every group in one pass (kdUnbind,
// kd.c:1299-1466; kdCellPot/kdSubPot/kdAddScoopPot, grav.c:8-135; the
// Hernquist-Katz spline SPLINE_POT, grav.h:11-31).
//
// Per group g (members in ascending iOrder, positions relative to rel and
// wrapped with half periods, kd.c:1341-1355):
//   pot_i = sum_{j != i} G m_j psi(r_ij, eps_i + eps_j)            (kdCellPot)
//         + sum_{ungrouped k within fScoop of the centre} G m_k psi  (scoop; the
//           reference applies it for every input type, kd.c:1379-1384)
//   then repeatedly: E_i = 1/2 |a (v_i - vcm) + aH (r_i - rcm)|^2 - pot_i (1+z);
//   if max E < 0 stop, else remove the first member with the largest E,
//   update rcm/vcm (FP64), swap it with the last member, and for pure dark
//   or pure star input subtract its potential from the others (kdSubPot).
//
// Potentials are accumulated in 64-bit fixed point (term * 2^S rounded to an
// integer).  The reference adds float terms into a double, which is exact
// for realistic groups, so when kdSubPot later subtracts the same terms the
// remainder is exact -- in particular a group's last member ends with
// potential exactly 0 (or its scoop part) and is unbound with E = 1/2 dv^2 >= 0.
// Integer sums reproduce that exactly and in any order.
//
// Kernels, every group in one launch each:
//  - scoop lists: one thread per group walks the tree of ungrouped particles;
//  - potentials: work items are the upper-triangle tile pairs (I <= J) of
//    every group, largest groups first; each pair's psi is evaluated once and
//    added to both ends (the terms are exact integers, so the sums do not
//    depend on the order);
//  - removal: one persistent kernel takes groups largest first from a queue:
//    groups above `tw` members get the whole block (BS threads, block-wide
//    arg-max with first-index ties), smaller groups one warp each (warp
//    shuffles only, no block barriers).
// (tw, BS) is picked by timing the candidates on the first call (autotune),
// or fixed through the context's options.  A per-group mode (one potential
// and one removal launch per group, the reference's serial loop on the GPU)
// serves as the unbatched comparison.
#include <algorithm>
#include <cfloat>
#include <vector>

#include <cooperative_groups.h>

#include "ctx.h"

namespace cg = cooperative_groups;

namespace skid {

namespace {

constexpr int POT_TILE = 128;   // power of two
// Every removal decision is the reference's: each pass computes FP32 energies
// with an error bound, and only members within twice the bound of the
// largest or smallest energy are evaluated exactly (the reference's FP64
// expression rounded to float, kd.c:1396-1399), so the arg-max and arg-min,
// ties included, are those of the reference's loop.  Groups up to this size
// use the plain FP32 form with a per-member bound; larger ones the staged
// a v + aH r form with one bound per pass (GB300's FP64 rate is a small
// fraction of its FP32 rate, so FP64 is kept to the few candidates).
constexpr int EXACT_E_MAX = 1024;

// The reference's pair factor, bit for bit.  grav.c:25-30 forms it as a float
// assigned from FP64 arithmetic (gcc, no contraction): Plummer
// 1.0/sqrt(d2 + 0.25*twoh*twoh); spline SPLINE_POT (grav.h:11-31) with
// r = sqrt(d2) in FP64, the polynomials evaluated left to right, and 1/r
// beyond the softening.  The FP64 forms below spell every operation out with
// round-to-nearest intrinsics so the compiler cannot fuse them.
__device__ __noinline__ float ref_dir_fp64(float d2f, float twohf, int plummer)
{
    const double r2 = (double)d2f, twoh = (double)twohf;
    if (plummer)
        return (float)__ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(r2, __dmul_rn(__dmul_rn(0.25, twoh), twoh))));
    const double r = __dsqrt_rn(r2);
    if (r < twoh) {
        const double dih = __ddiv_rn(2.0, twoh);
        const double u = __dmul_rn(r, dih);
        if (u < 1.0) {
            // dih*(7/5 - 2/3*u*u + 3/10*u*u*u*u - 1/10*u*u*u*u*u)
            const double a = __dmul_rn(__dmul_rn(2.0 / 3.0, u), u);
            const double b = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(3.0 / 10.0, u), u), u), u);
            const double c =
                __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(1.0 / 10.0, u), u), u), u), u);
            return (float)__dmul_rn(dih, __dsub_rn(__dadd_rn(__dsub_rn(7.0 / 5.0, a), b), c));
        }
        // -1/15*dir + dih*(8/5 - 4/3*u*u + u*u*u - 3/10*u*u*u*u + 1/30*u*u*u*u*u)
        const double dir = __ddiv_rn(1.0, r);
        const double a = __dmul_rn(__dmul_rn(4.0 / 3.0, u), u);
        const double b = __dmul_rn(__dmul_rn(u, u), u);
        const double c = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(3.0 / 10.0, u), u), u), u);
        const double e =
            __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(1.0 / 30.0, u), u), u), u), u);
        const double poly = __dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(8.0 / 5.0, a), b), c), e);
        return (float)__dadd_rn(__dmul_rn(-1.0 / 15.0, dir), __dmul_rn(dih, poly));
    }
    return (float)__ddiv_rn(1.0, r);
}

// 1/r beyond the softening as the reference rounds it: float(1.0/sqrt(d2)),
// two correctly rounded FP64 operations then a rounding to float.  That float
// is the one nearest the real 1/sqrt(d2) unless 1/sqrt(d2) lies within about
// 2^-52 (relative) of a midpoint between floats.  Here 1/sqrt(d2) is formed
// as the unevaluated float pair y + d, within 2^-43 of it: y the hardware
// reciprocal square root (within 2^-22) and d = y r / 2 one Newton
// correction, whose residual r = 1 - x y^2 comes from the error-free product
// x y = ph + pl (pl by a fused multiply-add) as fma(-pl, y, fma(-ph, y, 1)),
// each fused step rounding only the small result.  The float s nearest
// y + d is returned unless y + d lies within 2^-17 ulp(s) of a midpoint
// (|(y + d) - s|, exact by Dekker's fast two-sum, at or above
// (1/2 - 2^-17) ulp), or s is a power of two; those few pairs in a hundred
// thousand take the FP64 expression itself.
__device__ __forceinline__ float ref_rsqrt(float x)
{
    if (!(x >= 1e-30f && x <= 1e30f)) return ref_dir_fp64(x, 0.0f, 0);
    const float y = rsqrtf(x);
    const float ph = __fmul_rn(x, y);
    const float pl = __fmaf_rn(x, y, -ph);
    const float r = __fmaf_rn(-pl, y, __fmaf_rn(-ph, y, 1.0f));
    const float d = __fmul_rn(__fmul_rn(0.5f, y), r);
    const float s = __fadd_rn(y, d);
    const float e = __fsub_rn(d, __fsub_rn(s, y));
    const unsigned sb = __float_as_uint(s);
    // (1/2 - 2^-17) ulp(s): exponent of ulp/4, mantissa 2 - 2^-15
    const float near = __uint_as_float(((sb & 0x7f800000u) - (25u << 23)) | 0x7fff00u);
    if ((sb & 0x7fffffu) == 0u || fabsf(e) >= near) return ref_dir_fp64(x, 0.0f, 0);
    return s;
}

// Float-float numbers (an unevaluated sum h + l, |l| <= ulp(h) / 2) with
// round-to-nearest intrinsics throughout, so no step is contracted.  Every
// operation is within about 2^-46 (relative) of the real result.
struct ffl {
    float h, l;
};

__device__ __forceinline__ ffl ff_norm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ ffl ff_add(ffl a, ffl b)
{
    const float s = __fadd_rn(a.h, b.h);
    const float v = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return ff_norm(s, e);
}

__device__ __forceinline__ ffl ff_mul(ffl a, ffl b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ff_norm(p, e);
}

// A double constant as the nearest float pair (within 2^-48 of it).
#define SKID_FFC(x) ffl{(float)(x), (float)((x) - (double)(float)(x))}

// The spline branch of the reference's pair factor (grav.h:11-31 as
// grav.c:25-30 evaluates it, r < 2h) without FP64: the same real-number
// expression in float-float arithmetic, within about 2^-37 (relative) of
// its real value -- the one polynomial with cancellation has terms up to 16
// times its value -- while the reference's FP64 evaluation is within about
// 2^-45.  Both therefore round to the same float unless the value lies
// within 2^-32 (relative) of a midpoint between floats, or r is that close
// to 2h or u = 2r/(2h) to 1 (where the reference's own rounding could take
// the other branch).  Those inputs, tiny ones and powers of two return
// false, and the caller takes the FP64 expression.
__device__ __forceinline__ bool ref_spline_ff(float d2, float twoh, float &out)
{
    if (!(d2 >= 1e-30f && twoh >= 1e-30f && twoh <= 1e30f)) return false;
    // r = sqrt(d2): the correctly rounded root plus one Newton correction
    // (d2 - s^2 is exact by a fused multiply-add)
    const float s = __fsqrt_rn(d2);
    const ffl r = ff_norm(s, __fdiv_rn(__fmaf_rn(-s, s, d2), __fmul_rn(2.0f, s)));
    // the branch r < 2h, decided only when r is clear of 2h
    const float dr = ff_add(r, ffl{-twoh, 0.0f}).h;
    if (fabsf(dr) <= 0x1p-40f * twoh) return false;
    if (dr >= 0.0f) return false;   // 1/r beyond the softening: not this branch
    // dih = 2/(2h), the quotient plus its remainder (exact by a fused multiply-add)
    const float q = __fdiv_rn(2.0f, twoh);
    const ffl dih = ff_norm(q, __fdiv_rn(__fmaf_rn(-q, twoh, 2.0f), twoh));
    const ffl u = ff_mul(r, dih);
    const float du = __fadd_rn(__fsub_rn(u.h, 1.0f), u.l);
    if (fabsf(du) <= 0x1p-38f) return false;
    const ffl u2 = ff_mul(u, u);
    const ffl u4 = ff_mul(u2, u2);
    const ffl u5 = ff_mul(u4, u);
    ffl v;
    if (du < 0.0f) {
        // dih*(7/5 - 2/3 u^2 + 3/10 u^4 - 1/10 u^5)
        ffl p = ff_add(SKID_FFC(7.0 / 5.0), ff_mul(SKID_FFC(-2.0 / 3.0), u2));
        p = ff_add(p, ff_mul(SKID_FFC(3.0 / 10.0), u4));
        p = ff_add(p, ff_mul(SKID_FFC(-1.0 / 10.0), u5));
        v = ff_mul(dih, p);
    } else {
        // -1/15 / r + dih*(8/5 - 4/3 u^2 + u^3 - 3/10 u^4 + 1/30 u^5)
        const ffl u3 = ff_mul(u2, u);
        ffl p = ff_add(SKID_FFC(8.0 / 5.0), ff_mul(SKID_FFC(-4.0 / 3.0), u2));
        p = ff_add(p, u3);
        p = ff_add(p, ff_mul(SKID_FFC(-3.0 / 10.0), u4));
        p = ff_add(p, ff_mul(SKID_FFC(1.0 / 30.0), u5));
        // 1/r: the rounded reciprocal and its residual 1 - r y
        const float y = __frcp_rn(r.h);
        const float t = __fmaf_rn(-r.l, y, __fmaf_rn(-r.h, y, 1.0f));
        const ffl dir = ff_norm(y, __fmul_rn(y, t));
        v = ff_add(ff_mul(dih, p), ff_mul(SKID_FFC(-1.0 / 15.0), dir));
    }
    // the float nearest v, kept unless v is within 2^-9 ulp of a midpoint
    const float f = __fadd_rn(v.h, v.l);
    const float e = __fadd_rn(__fsub_rn(v.h, f), v.l);
    const unsigned fb = __float_as_uint(f);
    if (!(f >= 1e-30f && f <= 1e30f) || (fb & 0x7fffffu) == 0u) return false;
    // (1/2 - 2^-9) ulp(f): exponent of ulp/4, mantissa 2 - 2^-7
    const float near = __uint_as_float(((fb & 0x7f800000u) - (25u << 23)) | 0x7f0000u);
    if (fabsf(e) >= near) return false;
    out = f;
    return true;
}
#undef SKID_FFC

// The pair factor of every potential term, added (potentials, scoop) and
// subtracted (removal) alike, equal to the reference's float dir.  Beyond
// the softening (r >= 2h, certain once d2 clears (2h)^2 by the margin below)
// it is ref_rsqrt; inside, the float-float spline where it decides the
// rounding, else (and for Plummer softening) the FP64 form.
__device__ __forceinline__ float pair_dir(float d2, float twoh, int plummer)
{
    if (!plummer && d2 >= twoh * twoh * 1.000001f) return ref_rsqrt(d2);
    float v;
    if (!plummer && ref_spline_ff(d2, twoh, v)) return v;
    return ref_dir_fp64(d2, twoh, plummer);
}

__device__ __forceinline__ float wrap_h(float d, float h)
{
    // kd.c:1345-1350: if (dx > hx) dx -= 2*hx; if (dx <= -hx) dx += 2*hx
    if (d > h) d = fsub(d, fmul(2.0f, h));
    if (d <= -h) d = fadd(d, fmul(2.0f, h));
    return d;
}

// float -> int64 with round-half-to-even, bit-identical to __float2ll_rn for
// finite |f| < 2^63, on the integer units: the mantissa shifted by the
// exponent.  (GB300 runs the 64-bit conversion instructions on its FP64
// path, which made them the bottleneck of the potential sums.)
__device__ __forceinline__ long long f2ll_rn(float f)
{
    const unsigned b = __float_as_uint(f);
    const int e = (int)((b >> 23) & 0xffu);
    if (e == 0) return 0;                              // zero or denormal (< 0.5)
    const unsigned long long m = (b & 0x7fffffu) | 0x800000u;
    const int sh = e - 150;                            // |f| = m * 2^sh
    unsigned long long q;
    if (sh > 39) {
        q = 0x7fffffffffffffffull;                     // |f| >= 2^63: saturate
    } else if (sh >= 0) {
        q = m << sh;
    } else if (sh > -25) {
        const int r = -sh;                             // 1..24
        const unsigned long long rem = m & ((1ull << r) - 1ull);
        const unsigned long long half = 1ull << (r - 1);
        q = m >> r;
        q += (rem > half) || (rem == half && (q & 1ull));
    } else {
        q = 0;                                         // |f| < 0.5
    }
    return (b >> 31) ? -(long long)q : (long long)q;
}

// int64 -> float within two roundings (relative error <= 2^-23), on the
// FP32 and integer units: |p| in three 22-bit chunks, each exact as a float
// (2^23 + x - 2^23), recombined by two fused multiply-adds.
__device__ __forceinline__ float ll2f_approx(long long p)
{
    const unsigned long long a = p < 0 ? (unsigned long long)(-p) : (unsigned long long)p;
    const float c0 = __uint_as_float(0x4B000000u | (unsigned)(a & 0x3fffffull)) - 8388608.0f;
    const float c1 = __uint_as_float(0x4B000000u | (unsigned)((a >> 22) & 0x3fffffull)) - 8388608.0f;
    const float c2 = __uint_as_float(0x4B000000u | (unsigned)((a >> 44) & 0x3fffffull)) - 8388608.0f;
    const float f = __fmaf_rn(c2, 17592186044416.0f, __fmaf_rn(c1, 4194304.0f, c0));   // 2^44, 2^22
    return p < 0 ? -f : f;
}

// int64 -> float within three roundings (relative error below 2^-22), from
// the two 32-bit halves of |p| and one fused multiply-add: the FP32 energies
// of large groups only.
__device__ __forceinline__ float ll2f_fast(long long p)
{
    const unsigned long long a = p < 0 ? (unsigned long long)(-p) : (unsigned long long)p;
    const float f = __fmaf_rn(__uint2float_rn((unsigned)(a >> 32)), 4294967296.0f,
                              __uint2float_rn((unsigned)a));
    return p < 0 ? -f : f;
}

// Fixed-point quantum of a float term (scale = 2^S, exact multiply), equal to
// __float2ll_rn(t * scale).  Terms are non-negative: below 2^23 adding 2^23
// rounds to the nearest integer (ties to even) in the float adder, at or above
// it the float is already an integer, its mantissa shifted by the exponent.
__device__ __forceinline__ long long fx(float t, float scale)
{
    const float f = t * scale;
    if (f < 8388608.0f) {
        if (!(f >= 0.0f)) return f2ll_rn(f);          // negative or NaN: general form
        return (long long)(__float_as_uint(f + 8388608.0f) - 0x4B000000u);
    }
    const unsigned b = __float_as_uint(f);
    const int sh = (int)(b >> 23) - 150;              // 0 .. for f >= 2^23
    if (sh > 39) return f2ll_rn(f);                   // beyond 2^63: saturates
    return (long long)(((unsigned long long)((b & 0x7fffffu) | 0x800000u)) << sh);
}

__global__ void prep_members(const int *__restrict__ members, const int *__restrict__ gof, int n,
                             const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                             const skid_group *__restrict__ rec, float3 hP,
                             float4 *__restrict__ qr, float4 *__restrict__ qv)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int io = members[k];
        int g = gof[k];
        float4 p = pos4[io];
        const float *rel = rec[g].rel;
        qr[k] = make_float4(wrap_h(fsub(p.x, rel[0]), hP.x), wrap_h(fsub(p.y, rel[1]), hP.y),
                            wrap_h(fsub(p.z, rel[2]), hP.z), p.w);
        qv[k] = vel4[io];
    }
}

// Scoop: ungrouped particles within fScoop of each group's centre.
// pass 0 counts, pass 1 fills (offsets from an exclusive scan).
__global__ void scoop_kernel(TreeView t, const float *__restrict__ usoft,
                             const skid_group *__restrict__ rec, const int *__restrict__ gcount,
                             int ng, int nmax, float fBall2, float3 L, float3 hL, bool per,
                             int pass, int *__restrict__ cnt, const int *__restrict__ off,
                             float4 *__restrict__ list, float *__restrict__ lsoft)
{
    // every entry is written, group 0 (the ungrouped particles) with 0: the
    // counts are scanned into offsets as a whole
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int c = 0;
        int n = gcount[g];
        if (g > 0 && n > 0 && n < nmax && t.n > 0) {
            const float *cen = rec[g].rCenter;
            const float *rel = rec[g].rel;
            float3 q = make_float3(cen[0], cen[1], cen[2]);
            int o = pass ? off[g] : 0;
            int cp = 1;
            for (;;) {
                float4 blo = t.lo[cp], bhi = t.hi[cp];
                if (box_lb(q, blo, bhi, L, per) < fBall2) {
                    if (cp < t.leafBase) { cp <<= 1; continue; }
                    int b = (cp - t.leafBase) * SKID_LEAF, e = min(b + SKID_LEAF, t.n);
                    for (int j = b; j < e; ++j) {
                        float4 p = t.pos[j];
                        float d2 = d2of(img_dx(q.x, p.x, L.x, hL.x), img_dx(q.y, p.y, L.y, hL.y),
                                        img_dx(q.z, p.z, L.z, hL.z));
                        if (d2 < fBall2) {
                            if (pass) {
                                // grav.c:103-111
                                float nx = fsub(p.x, rel[0]), ny = fsub(p.y, rel[1]), nz = fsub(p.z, rel[2]);
                                if (nx > hL.x) nx = fsub(nx, L.x);
                                if (nx <= -hL.x) nx = fadd(nx, L.x);
                                if (ny > hL.y) ny = fsub(ny, L.y);
                                if (ny <= -hL.y) ny = fadd(ny, L.y);
                                if (nz > hL.z) nz = fsub(nz, L.z);
                                if (nz <= -hL.z) nz = fadd(nz, L.z);
                                list[o + c] = make_float4(nx, ny, nz, p.w);
                                lsoft[o + c] = usoft[j];
                            }
                            ++c;
                        }
                    }
                }
                cp = next_node(cp);
                if (cp == 1) break;
            }
        }
        if (!pass) cnt[g] = c;
    }
}


// ---- scheduling order: valid groups by descending size ----

__global__ void sched_keys(const int *__restrict__ gcount, int ng, int nmax, uint64_t *keys,
                           uint32_t *vals)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int n = gcount[g];
        bool ok = g > 0 && n > 0 && n < nmax;
        keys[g] = ok ? (uint64_t)(0x7fffffff - n) : 0xffffffffull;
        vals[g] = (uint32_t)g;
    }
}

// cnt[0] = valid groups, cnt[1] = groups above tw members
__global__ void sched_counts(const int *__restrict__ gcount, int ng, int nmax, int tw, int *cnt)
{
    int v = 0, b = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int n = gcount[g];
        if (g > 0 && n > 0 && n < nmax) {
            ++v;
            b += n > tw;
        }
    }
    for (int o = 16; o; o >>= 1) {
        v += __shfl_xor_sync(SKID_FULL, v, o);
        b += __shfl_xor_sync(SKID_FULL, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(cnt, v);
        atomicAdd(cnt + 1, b);
    }
}

// ---- potentials ----

// out[0]: groups taken by clusters, the largest ones above `floor` members
// but at most kmax of them; out[2]: the largest valid group's size (order is
// largest first)
__global__ void cluster_groups(const uint32_t *__restrict__ order, const int *d_nvalid,
                               const int *__restrict__ gcount, int floor, int kmax, int *out)
{
    if (threadIdx.x != 0) return;
    const int nv = *d_nvalid;
    int k = 0;
    while (k < nv && k < kmax && gcount[order[k]] > floor) ++k;
    out[0] = k;
    out[2] = nv > 0 ? gcount[order[0]] : 0;
}

__global__ void pot_nitems(const uint32_t *__restrict__ order, const int *d_nvalid,
                           const int *__restrict__ gcount, int ng, int *__restrict__ ni)
{
    int nv = *d_nvalid;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ng; k += gridDim.x * blockDim.x) {
        int c = 0;
        if (k < nv) {
            int nt = (gcount[order[k]] + POT_TILE - 1) / POT_TILE;
            c = nt * (nt + 1) / 2;
        }
        ni[k] = c;
    }
}

__global__ void pot_fill(const uint32_t *__restrict__ order, const int *d_nvalid,
                         const int *__restrict__ gcount, const int *__restrict__ ioff,
                         int2 *__restrict__ items)
{
    int nv = *d_nvalid;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += gridDim.x * blockDim.x) {
        int g = order[k];
        int nt = (gcount[g] + POT_TILE - 1) / POT_TILE;
        int o = ioff[k];
        for (int I = 0; I < nt; ++I)
            for (int J = I; J < nt; ++J) items[o++] = make_int2(g, (I << 16) | J);
    }
}

// One tile pair (I, J) of one group per block iteration, POT_TILE / 2
// threads with two rows each (t and t + POT_TILE / 2).  Off-diagonal items
// take every (i in I, j in J); diagonal items every i < j in the tile, plus
// the scoop terms of the tile's rows (kdAddScoopPot, grav.c:112-127).  At
// rotation step k thread t pairs its rows with column (t + k) mod T: the
// lanes of a warp touch distinct columns, so each warp keeps its own column
// accumulators (plain adds, a warp barrier per step), summed at the end.
// Columns carry G m 2^S, so a term is one multiply from its quantum.
constexpr int POT_THREADS = POT_TILE / 2;

struct PotRow {
    float4 r;     // position, G m 2^S
    float e;      // softening
    bool v;       // a member of the tile
};

// The terms of row a and column j (tr: on a, tc: on j).  far is at or above
// every pair's (2h)^2 (1 + 1e-6) in the tile pair (infinite for Plummer
// softening): beyond it pair_dir is 1/r, taken without forming the pair's
// softening, with the same value.
__device__ __forceinline__ void pot_pair(const PotRow &a, float4 rj, float ej, int plummer,
                                         float far, long long &tr, long long &tc)
{
    float d2 = d2of(fsub(a.r.x, rj.x), fsub(a.r.y, rj.y), fsub(a.r.z, rj.z));
    float dir = d2 >= far ? ref_rsqrt(d2) : pair_dir(d2, fadd(a.e, ej), plummer);
    tr = fx(fmul(rj.w, dir), 1.0f);
    // equal masses (all-dark runs): both ends get the same term
    tc = rj.w == a.r.w ? tr : fx(fmul(a.r.w, dir), 1.0f);
}

__global__ void __launch_bounds__(POT_THREADS)
pot_sym_kernel(const int2 *__restrict__ items, const int *d_nitems, int nitems_host,
               const int *__restrict__ gstart, const int *__restrict__ gcount,
               const float4 *__restrict__ qr, const float4 *__restrict__ qv,
               const int *__restrict__ soff, const int *__restrict__ scnt,
               const float4 *__restrict__ slist, const float *__restrict__ ssoft, float G,
               int plummer, float scale, long long *__restrict__ pot)
{
    constexpr int T = POT_TILE, H = POT_TILE / 2, NW = POT_THREADS / 32;
    __shared__ float4 sr[T];
    __shared__ float ss[T];
    __shared__ long long acc_w[NW][T];
    __shared__ float emax_w[2][NW];
    const int t = threadIdx.x, wid = t >> 5;
    const int nitems = nitems_host >= 0 ? nitems_host : *d_nitems;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        int2 w = items[it];
        int g = w.x, I = w.y >> 16, J = w.y & 0xffff;
        int s = gstart[g], n = gcount[g];
        PotRow ra, rb;
        {
            const int ia = I * T + t, ib = ia + H;
            ra.v = ia < n;
            rb.v = ib < n;
            float4 q = ra.v ? qr[s + ia] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            ra.r = make_float4(q.x, q.y, q.z, fmul(G, q.w) * scale);
            ra.e = ra.v ? qv[s + ia].w : 0.0f;
            q = rb.v ? qr[s + ib] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            rb.r = make_float4(q.x, q.y, q.z, fmul(G, q.w) * scale);
            rb.e = rb.v ? qv[s + ib].w : 0.0f;
        }
        int j0 = J * T;
        int nj = min(T, n - j0);
        __syncthreads();
        for (int c = t; c < T; c += POT_THREADS) {
            if (c < nj) {
                float4 q = qr[s + j0 + c];
                sr[c] = make_float4(q.x, q.y, q.z, fmul(G, q.w) * scale);
                ss[c] = qv[s + j0 + c].w;
            }
#pragma unroll
            for (int k = 0; k < NW; ++k) acc_w[k][c] = 0;
        }
        __syncthreads();
        // the far bound: (largest row softening + largest column softening)^2,
        // above every pair's own (softenings are non-negative, so their bit
        // patterns order like their values)
        float far = INFINITY;
        if (!plummer) {
            float er = fmaxf(ra.v ? ra.e : 0.0f, rb.v ? rb.e : 0.0f), ec = 0.0f;
            for (int c = t; c < nj; c += POT_THREADS) ec = fmaxf(ec, ss[c]);
            er = __uint_as_float(__reduce_max_sync(SKID_FULL, __float_as_uint(er)));
            ec = __uint_as_float(__reduce_max_sync(SKID_FULL, __float_as_uint(ec)));
            if ((t & 31) == 0) {
                emax_w[0][wid] = er;
                emax_w[1][wid] = ec;
            }
            __syncthreads();
            er = emax_w[0][0];
            ec = emax_w[1][0];
#pragma unroll
            for (int k = 1; k < NW; ++k) {
                er = fmaxf(er, emax_w[0][k]);
                ec = fmaxf(ec, emax_w[1][k]);
            }
            const float twoh = er + ec;
            far = twoh * twoh * 1.000001f;
        }
        long long acca = 0, accb = 0;
        if (I != J) {
            for (int k = 0; k < T; ++k) {
                const int jl = (t + k) & (T - 1);
                if (jl < nj) {
                    const float4 rj = sr[jl];
                    const float ej = ss[jl];
                    long long tr, tc, col = 0;
                    if (ra.v) { pot_pair(ra, rj, ej, plummer, far, tr, tc); acca += tr; col += tc; }
                    if (rb.v) { pot_pair(rb, rj, ej, plummer, far, tr, tc); accb += tr; col += tc; }
                    acc_w[wid][jl] += col;
                }
                __syncwarp();
            }
        } else {
            // offset (column - row) mod T in 1..T/2 for row t (k = 1..H),
            // 1..T/2-1 for row t + H (k = H+1..T-1): each pair once
            for (int k = 1; k < T; ++k) {
                const int jl = (t + k) & (T - 1);
                const PotRow &a = k <= H ? ra : rb;
                if (jl < nj && a.v) {
                    long long tr, tc;
                    pot_pair(a, sr[jl], ss[jl], plummer, far, tr, tc);
                    if (k <= H) acca += tr; else accb += tr;
                    acc_w[wid][jl] += tc;
                }
                __syncwarp();
            }
            int so = soff[g], sc = scnt[g];
            for (int jb = 0; jb < sc; jb += T) {
                __syncthreads();
                for (int c = t; c < T; c += POT_THREADS)
                    if (jb + c < sc) {
                        float4 q = slist[so + jb + c];
                        sr[c] = make_float4(q.x, q.y, q.z, fmul(G, q.w) * scale);
                        ss[c] = ssoft[so + jb + c];
                    }
                __syncthreads();
                int cnt = min(T, sc - jb);
                for (int k = 0; k < cnt; ++k) {
                    const float4 rj = sr[k];
                    const float ej = ss[k];
                    // kdAddScoopPot's pair: d2 from the scoop particle
                    float d2a = d2of(fsub(rj.x, ra.r.x), fsub(rj.y, ra.r.y), fsub(rj.z, ra.r.z));
                    float d2b = d2of(fsub(rj.x, rb.r.x), fsub(rj.y, rb.r.y), fsub(rj.z, rb.r.z));
                    if (ra.v) acca += fx(fmul(rj.w, pair_dir(d2a, fadd(ej, ra.e), plummer)), 1.0f);
                    if (rb.v) accb += fx(fmul(rj.w, pair_dir(d2b, fadd(ej, rb.e), plummer)), 1.0f);
                }
            }
        }
        __syncthreads();
        if (ra.v) atomicAdd((unsigned long long *)&pot[s + I * T + t], (unsigned long long)acca);
        if (rb.v) atomicAdd((unsigned long long *)&pot[s + I * T + t + H], (unsigned long long)accb);
        for (int c = t; c < nj; c += POT_THREADS) {
            long long cs = 0;
#pragma unroll
            for (int k = 0; k < NW; ++k) cs += acc_w[k][c];
            if (cs) atomicAdd((unsigned long long *)&pot[s + j0 + c], (unsigned long long)cs);
        }
    }
}

// ---- removal ----

struct ArgRed {
    float v;
    int i;
};

__device__ __forceinline__ ArgRed warp_argmax(ArgRed a)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        float v = __shfl_xor_sync(SKID_FULL, a.v, o);
        int i = __shfl_xor_sync(SKID_FULL, a.i, o);
        if (v > a.v || (v == a.v && i < a.i)) { a.v = v; a.i = i; }
    }
    return a;
}

__device__ __forceinline__ ArgRed warp_argmin(ArgRed a)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        float v = __shfl_xor_sync(SKID_FULL, a.v, o);
        int i = __shfl_xor_sync(SKID_FULL, a.i, o);
        if (v < a.v || (v == a.v && i < a.i)) { a.v = v; a.i = i; }
    }
    return a;
}

// A thread's two largest (a, then b) or two smallest energies, the first
// index kept on ties (members are visited in increasing index).
__device__ __forceinline__ void keep_top2(ArgRed &a, ArgRed &b, float E, int i)
{
    if (E > a.v) { b = a; a.v = E; a.i = i; }
    else if (E > b.v) { b.v = E; b.i = i; }
}

__device__ __forceinline__ void keep_bot2(ArgRed &a, ArgRed &b, float E, int i)
{
    if (E < a.v) { b = a; a.v = E; a.i = i; }
    else if (E < b.v) { b.v = E; b.i = i; }
}

struct RemoveArgs {
    const int *gstart, *gcount;
    int ng, nmax;
    float4 *qr, *qv;
    float4 *qw;                     // large groups' staged a v + aH r (w: softening)
    int *qid;
    long long *pot;
    skid_group *rec;
    int *grp;
    int *d_unbound;
    float G, fShift, fCosmo, opz;   // a, a*H(a), 1+z
    float z;
    float scale, inv_scale;         // 2^S, 2^-S
    float3 hP;
    int plummer, subpot, nounbind;
    const uint32_t *order;          // valid groups, largest first
    const int *d_cnt;               // [valid groups, groups above tw]
    int *d_queue;
    const int *d_ccnt;              // groups taken by clusters (the largest, a prefix of order)
    int *d_cqueue;
    int qcap;                       // members per block slice a cluster can hold
    int single;                     // > 0: process only this group (per-group mode)
};

// E_i of kd.c:1392-1400: exact form (the reference's FP64 expression with
// each operation rounded as gcc rounds it, no fused multiply-adds, then
// rounded to float) or FP32 form.  Exact form:
//   dv_j = (float)(a * ((double)v_j - vcm_j) + aH * ((double)r_j - rcm_j))
//   dv2  = dv_0^2 + dv_1^2 + dv_2^2                      (float)
//   E    = (float)(0.5 * dv2 - pot * (1.0 + z))
__device__ __forceinline__ float exact_energy(const RemoveArgs &A, float4 r, float4 v, long long p,
                                              const double *dcm, double inv_d, double opz_d)
{
    const double fs = A.fShift, fc = A.fCosmo;
    const float dv0 = (float)__dadd_rn(__dmul_rn(fs, __dsub_rn((double)v.x, dcm[3])),
                                       __dmul_rn(fc, __dsub_rn((double)r.x, dcm[0])));
    const float dv1 = (float)__dadd_rn(__dmul_rn(fs, __dsub_rn((double)v.y, dcm[4])),
                                       __dmul_rn(fc, __dsub_rn((double)r.y, dcm[1])));
    const float dv2 = (float)__dadd_rn(__dmul_rn(fs, __dsub_rn((double)v.z, dcm[5])),
                                       __dmul_rn(fc, __dsub_rn((double)r.z, dcm[2])));
    const float dd = fadd(fadd(fmul(dv0, dv0), fmul(dv1, dv1)), fmul(dv2, dv2));
    // pot * 2^-S is exact (a power-of-two scale of an integer below 2^53)
    return (float)__dsub_rn(__dmul_rn(0.5, (double)dd), __dmul_rn(__dmul_rn((double)p, inv_d), opz_d));
}

__device__ __forceinline__ float member_energy(bool exact, const RemoveArgs &A, float4 r, float4 v,
                                               long long p, const double *dcm, const float *scm,
                                               double inv_d, double opz_d)
{
    if (exact) return exact_energy(A, r, v, p, dcm, inv_d, opz_d);
    float dv0 = A.fShift * (v.x - scm[3]) + A.fCosmo * (r.x - scm[0]);
    float dv1 = A.fShift * (v.y - scm[4]) + A.fCosmo * (r.y - scm[1]);
    float dv2 = A.fShift * (v.z - scm[5]) + A.fCosmo * (r.z - scm[2]);
    float dd = fadd(fadd(fmul(dv0, dv0), fmul(dv1, dv1)), fmul(dv2, dv2));
    return 0.5f * dd - (ll2f_approx(p) * A.inv_scale) * A.opz;
}

// Bound on |FP32 energy - exact energy|: each of them is within a few
// roundings of the real value of the same expression, so 2^-19 of the sum of
// the magnitudes that enter it (velocity and position terms before their
// cancellation, the kinetic term, the potential term) bounds the difference.
__device__ __forceinline__ float energy_err(const RemoveArgs &A, float4 r, float4 v, long long p,
                                            const float *scm, float e32)
{
    const float a = fabsf(A.fShift), c = fabsf(A.fCosmo);
    float s = 0.0f, k = 0.0f;
    const float vv[3] = {v.x, v.y, v.z}, rr[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float mag = a * (fabsf(vv[d]) + fabsf(scm[3 + d])) + c * (fabsf(rr[d]) + fabsf(scm[d]));
        float dv = A.fShift * (vv[d] - scm[3 + d]) + A.fCosmo * (rr[d] - scm[d]);
        s += mag * (2.0f * fabsf(dv) + mag);
        k += dv * dv;
    }
    float pe = fabsf(ll2f_approx(p) * A.inv_scale * A.opz);
    return 1.9073486e-06f * (s + k + pe + fabsf(e32)) + 1e-30f;   // 2^-19
}

// kdSubPot (grav.c:44-59) of the removed particle rs on member (r, v).
__device__ __forceinline__ long long sub_pot(const RemoveArgs &A, float4 rs, float es, float4 r,
                                             float4 v, long long p)
{
    float d2 = d2of(fsub(rs.x, r.x), fsub(rs.y, r.y), fsub(rs.z, r.z));
    float dir = pair_dir(d2, fadd(es, v.w), A.plummer);
    return p - fx(fmul(fmul(A.G, rs.w) * A.scale, dir), 1.0f);
}

// centre of mass after removing (r, v): kd.c:1424-1431,
//   dMass -= m;  rcm_j += m/dMass * (rcm_j - r_j);  vcm_j likewise,
// each FP64 operation rounded separately as the reference's are.
__device__ __forceinline__ void rcm_update(double &mass, double *dcm, float4 r, float4 v)
{
    mass = __dsub_rn(mass, (double)r.w);
    const double f = __ddiv_rn((double)r.w, mass);
    const float x[6] = {r.x, r.y, r.z, v.x, v.y, v.z};
#pragma unroll
    for (int d = 0; d < 6; ++d)
        dcm[d] = __dadd_rn(dcm[d], __dmul_rn(f, __dsub_rn(dcm[d], (double)x[d])));
}

__device__ __forceinline__ void write_record(const RemoveArgs &A, int g, int n, double mass,
                                             const double *dcm, float4 rb, int nrem)
{
    skid_group r = A.rec[g];
    r.nMembers = n;
    r.fMass = (float)mass;
    r.vcm[0] = (float)dcm[3];
    r.vcm[1] = (float)dcm[4];
    r.vcm[2] = (float)dcm[5];
    float hx = A.hP.x;   // kd.c:1452-1456 wraps every axis with hx
    r.rBound[0] = wrap_h(fadd(rb.x, r.rel[0]), hx);
    r.rBound[1] = wrap_h(fadd(rb.y, r.rel[1]), hx);
    r.rBound[2] = wrap_h(fadd(rb.z, r.rel[2]), hx);
    A.rec[g] = r;
    if (nrem) atomicAdd(A.d_unbound, nrem);
}

// A small group, one warp: every lane keeps the FP64 centre itself (the same
// values on every lane), lane 0 writes.
__device__ void warp_group(const RemoveArgs &A, int g)
{
    const int lane = threadIdx.x & 31;
    const int s = A.gstart[g], n0 = A.gcount[g];
    float4 *qr = A.qr + s;
    float4 *qv = A.qv + s;
    int *qid = A.qid + s;
    long long *pot = A.pot + s;
    double m = 0.0, dcm[6] = {0, 0, 0, 0, 0, 0};
    for (int i = lane; i < n0; i += 32) {
        float4 r = qr[i], v = qv[i];
        m += r.w;
        dcm[0] += fmul(r.w, r.x); dcm[1] += fmul(r.w, r.y); dcm[2] += fmul(r.w, r.z);
        dcm[3] += fmul(r.w, v.x); dcm[4] += fmul(r.w, v.y); dcm[5] += fmul(r.w, v.z);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        m += __shfl_xor_sync(SKID_FULL, m, o);
        for (int d = 0; d < 6; ++d) dcm[d] += __shfl_xor_sync(SKID_FULL, dcm[d], o);
    }
    float scm[6];
    for (int d = 0; d < 6; ++d) {
        dcm[d] /= m;
        scm[d] = (float)dcm[d];
    }
    const bool exact = n0 <= EXACT_E_MAX;
    const double opz_d = 1.0 + (double)A.z, inv_d = 1.0 / (double)A.scale;
    int n = n0, nrem = 0, imin = 0;
    bool have = false;
    float4 rs = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float es = 0.0f;
    for (;;) {
        ArgRed mx{-FLT_MAX, 0x7fffffff}, mn{FLT_MAX, 0x7fffffff};
        ArgRed mx2 = mx, mn2 = mn;
        // FP32 energies with error bounds
        float dmax = 0.0f;
        for (int i = lane; i < n; i += 32) {
            float4 r = qr[i], v = qv[i];
            long long p = pot[i];
            if (have && A.subpot) {
                p = sub_pot(A, rs, es, r, v, p);
                pot[i] = p;
            }
            float E = member_energy(false, A, r, v, p, dcm, scm, inv_d, opz_d);
            keep_top2(mx, mx2, E, i);
            keep_bot2(mn, mn2, E, i);
            if (exact) dmax = fmaxf(dmax, energy_err(A, r, v, p, scm, E));
        }
        float hi = 0.0f, lo = 0.0f;
        const ArgRed t1 = mx, b1 = mn;
        // members again, in the same order with the same FP32 energies: the
        // candidates on the asked sides exactly (FP64, as the reference)
        auto rescan = [&](bool scan_hi, bool scan_lo) {
            for (int i = lane; i < n; i += 32) {
                float4 r = qr[i], v = qv[i];
                long long p = pot[i];
                float E = member_energy(false, A, r, v, p, dcm, scm, inv_d, opz_d);
                const bool ch = scan_hi && E >= hi, cl = scan_lo && E <= lo;
                if (ch || cl) {
                    float X = member_energy(true, A, r, v, p, dcm, scm, inv_d, opz_d);
                    if (ch && X > mx.v) { mx.v = X; mx.i = i; }
                    if (cl && X < mn.v) { mn.v = X; mn.i = i; }
                }
            }
        };
        if (exact) {
            // only members whose FP32 energy is within twice the error bound
            // of the extremes can be the exact arg-max / arg-min
            float emax = mx.v, emin = mn.v;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                emax = fmaxf(emax, __shfl_xor_sync(SKID_FULL, emax, o));
                emin = fminf(emin, __shfl_xor_sync(SKID_FULL, emin, o));
                dmax = fmaxf(dmax, __shfl_xor_sync(SKID_FULL, dmax, o));
            }
            hi = emax - 2.0f * dmax;
            lo = emin + 2.0f * dmax;
            // One candidate alone is the exact arg-max (every other member's
            // exact energy is below emax - dmax, and its own at least that),
            // and the sign of its exact energy is known when its FP32 energy
            // is at least the bound, or below minus the bound: the usual pass
            // needs no FP64 energy.  Otherwise the candidates are evaluated
            // exactly -- usually just the lane's own extreme, else its
            // members again.
            const unsigned chi = __ballot_sync(SKID_FULL, t1.v >= hi);
            const bool one = chi != 0 && (chi & (chi - 1)) == 0 && !__any_sync(SKID_FULL, mx2.v >= hi);
            if (one && emax >= dmax) {
                mx.v = emax;
                mx.i = __shfl_sync(SKID_FULL, t1.i, __ffs(chi) - 1);
            } else if (one && emax < -dmax) {
                mx.v = emax;
            } else {
                mx = ArgRed{-FLT_MAX, 0x7fffffff};
                if (t1.i < n && t1.v >= hi && mx2.v < hi) {
                    mx.v = member_energy(true, A, qr[t1.i], qv[t1.i], pot[t1.i], dcm, scm, inv_d, opz_d);
                    mx.i = t1.i;
                }
                if (mx2.v >= hi) rescan(true, false);
                mx = warp_argmax(mx);
            }
        } else {
            mx = warp_argmax(mx);
        }
        if (!(mx.v >= 0.0f) || A.nounbind || n == 0) {
            // the group's most bound member (kd.c:1389-1409: fTotMin starts
            // at 1), needed only once the removals stop
            if (exact) {
                mn = ArgRed{FLT_MAX, 0x7fffffff};
                if (b1.i < n && b1.v <= lo && mn2.v > lo) {
                    mn.v = member_energy(true, A, qr[b1.i], qv[b1.i], pot[b1.i], dcm, scm, inv_d, opz_d);
                    mn.i = b1.i;
                }
                if (mn2.v <= lo) rescan(false, true);
            }
            mn = warp_argmin(mn);
            imin = mn.v < 1.0f ? mn.i : 0;
            break;
        }
        const int ib = mx.i;
        __syncwarp();
        float4 r = qr[ib], v = qv[ib];
        __syncwarp();   // every lane has read the removed member before lane 0 swaps it away
        if (lane == 0) A.grp[qid[ib]] = 0;
        ++nrem;
        const int nn = n - 1;
        if (nn == 0) {
            m = 0.0;
            dcm[3] = dcm[4] = dcm[5] = 0.0;
            n = 0;
            break;
        }
        rcm_update(m, dcm, r, v);
        for (int d = 0; d < 6; ++d) scm[d] = (float)dcm[d];
        if (lane == 0) {
            // swap with the last member (kd.c:1435-1440)
            float4 rl = qr[nn], vl = qv[nn];
            int il = qid[nn], ir = qid[ib];
            long long pl = pot[nn], pb = pot[ib];
            qr[ib] = rl; qv[ib] = vl; qid[ib] = il; pot[ib] = pl;
            qr[nn] = r; qv[nn] = v; qid[nn] = ir; pot[nn] = pb;
        }
        __syncwarp();
        rs = r;
        es = v.w;
        have = true;
        n = nn;
    }
    __syncwarp();
    if (lane == 0) write_record(A, g, n, m, dcm, qr[imin], nrem);
    __syncwarp();
}

template <int BS>
struct BlockShared {
    ArgRed smax[BS / 32], smin[BS / 32];
    float4 s_r;
    float s_eps;
    float s_cm[6];
    int s_n, s_go, s_have, s_imin, s_item;
    double d_cm[6], d_mass;
    double part[BS / 32][7];
    float ext[BS / 32][4];      // per-warp FP32 energy max, min, error-bound terms
    float s_w[3];               // a vcm + aH rcm (large groups' FP32 energies)
    float s_mW;                 // max_j |a vcm_j| + |aH rcm_j|
    float s_mg;                 // max over members and axes of |a v_j| + |aH r_j|
    float gpart[8][4];          // a cluster's blocks' partials, gathered (rank order)
    ArgRed gmx[8], gmn[8];
    int ccnt[BS / 32];          // per-warp arg-max candidate counts (two for a thread with two)
    int cidx[BS / 32];          // the warp's first candidate
    // records of each warp's first candidate (slot BS/32: the removed member
    // when the decision needed the exact energies)
    float4 cr[BS / 32 + 1], cv[BS / 32 + 1], cw[BS / 32 + 1];
    long long cp[BS / 32 + 1];
    int cid[BS / 32 + 1];
};

// max_j |a c_j| + |aH c_{j-3}| of a centre (rcm, vcm)
__device__ __forceinline__ float centre_mag(const RemoveArgs &A, const double *dcm)
{
    float m = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        m = fmaxf(m, fabsf(A.fShift * (float)dcm[3 + d]) + fabsf(A.fCosmo * (float)dcm[d]));
    return m * 1.0000002f;
}

// FP32 filter energy of a large group's member from its staged
// w = a v + aH r: E = 1/2 |w - W|^2 - pot (1+z) 2^-S (dd and pe returned for
// the pass's error bound), each operation rounded as written, so every
// evaluation of a member gives the same value.
__device__ __forceinline__ float staged_energy(float4 w, long long p, float wx, float wy, float wz,
                                              float epot, float &dd, float &pe)
{
    const float dx = __fsub_rn(w.x, wx), dy = __fsub_rn(w.y, wy), dz = __fsub_rn(w.z, wz);
    dd = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    pe = __fmul_rn(ll2f_fast(p), epot);
    return __fsub_rn(__fmul_rn(0.5f, dd), pe);
}

// A large group, the whole block.
template <int BS>
__device__ void block_group(const RemoveArgs &A, int g, BlockShared<BS> &S)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int s = A.gstart[g], n0 = A.gcount[g];
    float4 *qr = A.qr + s;
    float4 *qv = A.qv + s;
    int *qid = A.qid + s;
    long long *pot = A.pot + s;
    double m = 0.0, c[6] = {0, 0, 0, 0, 0, 0};
    for (int i = tid; i < n0; i += BS) {
        float4 r = qr[i], v = qv[i];
        m += r.w;
        c[0] += fmul(r.w, r.x); c[1] += fmul(r.w, r.y); c[2] += fmul(r.w, r.z);
        c[3] += fmul(r.w, v.x); c[4] += fmul(r.w, v.y); c[5] += fmul(r.w, v.z);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        m += __shfl_xor_sync(SKID_FULL, m, o);
        for (int d = 0; d < 6; ++d) c[d] += __shfl_xor_sync(SKID_FULL, c[d], o);
    }
    __syncthreads();
    if (lane == 0) {
        S.part[w][0] = m;
        for (int d = 0; d < 6; ++d) S.part[w][1 + d] = c[d];
    }
    __syncthreads();
    if (tid == 0) {
        // warp partials in warp order: the same sums on every run
        double t[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < BS / 32; ++k)
            for (int d = 0; d < 7; ++d) t[d] += S.part[k][d];
        S.d_mass = t[0];
        for (int d = 0; d < 6; ++d) {
            S.d_cm[d] = t[1 + d] / t[0];
            S.s_cm[d] = (float)S.d_cm[d];
        }
        S.s_n = n0;
        S.s_have = 0;
        S.s_go = 1;
        S.s_imin = 0;
        for (int d = 0; d < 3; ++d)
            S.s_w[d] = (float)((double)A.fShift * S.d_cm[3 + d] + (double)A.fCosmo * S.d_cm[d]);
    }
    __syncthreads();
    int nrem = 0;
    const bool exact = n0 <= EXACT_E_MAX;
    const double opz_d = 1.0 + (double)A.z, inv_d = 1.0 / (double)A.scale;
    float4 *qw = A.qw + s;
    if (!exact) {
        // FP32 filter energies E_i = 1/2 |w_i - W|^2 - pot_i (1+z), with
        // w_i = a v_i + aH r_i fixed per member and W = a vcm + aH rcm per
        // pass; their error bound needs the largest |a v_j| + |aH r_j|
        float mg = 0.0f;
        for (int i = tid; i < n0; i += BS) {
            float4 r = qr[i], v = qv[i];
            qw[i] = make_float4(__fmaf_rn(A.fShift, v.x, A.fCosmo * r.x),
                                __fmaf_rn(A.fShift, v.y, A.fCosmo * r.y),
                                __fmaf_rn(A.fShift, v.z, A.fCosmo * r.z), v.w);
            mg = fmaxf(mg, fabsf(A.fShift * v.x) + fabsf(A.fCosmo * r.x));
            mg = fmaxf(mg, fabsf(A.fShift * v.y) + fabsf(A.fCosmo * r.y));
            mg = fmaxf(mg, fabsf(A.fShift * v.z) + fabsf(A.fCosmo * r.z));
        }
        mg = __uint_as_float(__reduce_max_sync(SKID_FULL, __float_as_uint(mg)));
        if (lane == 0) S.ext[w][0] = mg;
        __syncthreads();
        if (tid == 0) {
            float t = 0.0f;
            for (int k = 0; k < BS / 32; ++k) t = fmaxf(t, S.ext[k][0]);
            S.s_mg = t * 1.0000002f;
            S.s_mW = centre_mag(A, S.d_cm);
        }
        __syncthreads();
    }
    const float epot = A.inv_scale * A.opz;
    for (;;) {
        const int n = S.s_n;
        const bool have = S.s_have != 0;
        const float4 rs = S.s_r;
        const float es = S.s_eps;
        double dcm[6];
        float scm[6];
        for (int d = 0; d < 6; ++d) { dcm[d] = S.d_cm[d]; scm[d] = S.s_cm[d]; }
        const float wx = S.s_w[0], wy = S.s_w[1], wz = S.s_w[2];
        // the thread's two largest and two smallest FP32 energies (first
        // index first on ties), the block's extremes, and the pass's bound
        // on |FP32 energy - reference energy| (bnd)
        ArgRed mx{-FLT_MAX, 0x7fffffff}, mn{FLT_MAX, 0x7fffffff};
        ArgRed x2 = mx, n2 = mn;
        float gmax = -FLT_MAX, gmin = FLT_MAX, bnd = 0.0f;
        // The lane holding its warp's largest FP32 energy (the only lane of
        // the warp that can hold the member removed in the usual pass)
        // prefetches that member's records into L1 while the block meets at
        // the barrier.
        auto prefetch_top = [&](float wmax) {
            if (mx.v == wmax && mx.i < n) {
                asm volatile("prefetch.global.L1 [%0];" ::"l"(qr + mx.i));
                asm volatile("prefetch.global.L1 [%0];" ::"l"(qv + mx.i));
                asm volatile("prefetch.global.L1 [%0];" ::"l"(pot + mx.i));
                asm volatile("prefetch.global.L1 [%0];" ::"l"(qid + mx.i));
                if (!exact) asm volatile("prefetch.global.L1 [%0];" ::"l"(qw + mx.i));
            }
        };
        if (exact) {
            float dmax = 0.0f;
            for (int i = tid; i < n; i += BS) {
                float4 r = qr[i], v = qv[i];
                long long p = pot[i];
                if (have && A.subpot) {
                    p = sub_pot(A, rs, es, r, v, p);
                    pot[i] = p;
                }
                float E = member_energy(false, A, r, v, p, dcm, scm, inv_d, opz_d);
                keep_top2(mx, x2, E, i);
                keep_bot2(mn, n2, E, i);
                dmax = fmaxf(dmax, energy_err(A, r, v, p, scm, E));
            }
            float a0 = mx.v, a1 = mn.v;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                a0 = fmaxf(a0, __shfl_xor_sync(SKID_FULL, a0, o));
                a1 = fminf(a1, __shfl_xor_sync(SKID_FULL, a1, o));
                dmax = fmaxf(dmax, __shfl_xor_sync(SKID_FULL, dmax, o));
            }
            prefetch_top(a0);
            if (lane == 0) {
                S.ext[w][0] = a0;
                S.ext[w][1] = a1;
                S.ext[w][2] = dmax;
            }
            __syncthreads();
            for (int k = 0; k < BS / 32; ++k) {
                gmax = fmaxf(gmax, S.ext[k][0]);
                gmin = fminf(gmin, S.ext[k][1]);
                bnd = fmaxf(bnd, S.ext[k][2]);
            }
        } else {
            const float gms = fmul(A.G, rs.w) * A.scale;   // the removed member's G m 2^S
            const bool sub = have && A.subpot;
            float ddmx = 0.0f, pemx = 0.0f;
            // RB members per thread per batch, all loaded before any is used,
            // so their memory latencies overlap
            constexpr int RB = BS >= 1024 ? 2 : 4;
            for (int i0 = tid; i0 < n; i0 += RB * BS) {
                float4 r[RB], wv[RB];
                long long p[RB];
#pragma unroll
                for (int k = 0; k < RB; ++k) {
                    const int i = i0 + k * BS;
                    if (i < n) { r[k] = qr[i]; wv[k] = qw[i]; p[k] = pot[i]; }
                }
#pragma unroll
                for (int k = 0; k < RB; ++k) {
                    const int i = i0 + k * BS;
                    if (i >= n) break;
                    if (sub) {
                        // kdSubPot (grav.c:44-59): the term the potentials added
                        float d2 = d2of(fsub(rs.x, r[k].x), fsub(rs.y, r[k].y), fsub(rs.z, r[k].z));
                        p[k] -= fx(fmul(gms, pair_dir(d2, fadd(es, wv[k].w), A.plummer)), 1.0f);
                        pot[i] = p[k];
                    }
                    float dd, pe;
                    const float E = staged_energy(wv[k], p[k], wx, wy, wz, epot, dd, pe);
                    keep_top2(mx, x2, E, i);
                    keep_bot2(mn, n2, E, i);
                    ddmx = fmaxf(ddmx, dd);
                    pemx = fmaxf(pemx, fabsf(pe));
                }
            }
            // Bound on |E_i(FP32) - E_i(reference)|: with C = max |a v| +
            // |aH r| over members plus the same for the centre, each
            // component of w_i - W is within 2^-21 C of the reference's dv,
            // so 2^-19 (C (sqrt(3 dd) + 3 C) + 1.5 dd + 2 |pe|) over the
            // pass's largest dd and |pe| covers every member, several times
            // over.
            float a0 = mx.v, a1 = mn.v;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                a0 = fmaxf(a0, __shfl_xor_sync(SKID_FULL, a0, o));
                a1 = fminf(a1, __shfl_xor_sync(SKID_FULL, a1, o));
                ddmx = fmaxf(ddmx, __shfl_xor_sync(SKID_FULL, ddmx, o));
                pemx = fmaxf(pemx, __shfl_xor_sync(SKID_FULL, pemx, o));
            }
            prefetch_top(a0);
            if (lane == 0) {
                S.ext[w][0] = a0;
                S.ext[w][1] = a1;
                S.ext[w][2] = ddmx;
                S.ext[w][3] = pemx;
            }
            __syncthreads();
            float gdd = 0.0f, gpe = 0.0f;
            for (int k = 0; k < BS / 32; ++k) {
                gmax = fmaxf(gmax, S.ext[k][0]);
                gmin = fminf(gmin, S.ext[k][1]);
                gdd = fmaxf(gdd, S.ext[k][2]);
                gpe = fmaxf(gpe, S.ext[k][3]);
            }
            const float C = S.s_mg + S.s_mW;
            bnd = 1.9073486e-06f * (C * (1.7320509f * sqrtf(gdd) + 3.0f * C) + 1.5f * gdd + 2.0f * gpe) +
                  1e-30f;
        }
        // Only members within twice the bound of the extremes can be the
        // exact arg-max or arg-min.
        const float hi = gmax - 2.0f * bnd, lo = gmin + 2.0f * bnd;
        const ArgRed t1 = mx, b1 = mn;
        // the last member's records, final for this pass now (their owners
        // wrote the potentials before the barrier), for the swap
        float4 lr = make_float4(0.0f, 0.0f, 0.0f, 0.0f), lv = lr, lw = lr;
        long long lp = 0;
        int lq = 0;
        if (tid == 32 && n > 1) {
            lr = qr[n - 1];
            lv = qv[n - 1];
            lp = pot[n - 1];
            lq = qid[n - 1];
            if (!exact) lw = qw[n - 1];
        }
        // members again, in the same order with the same FP32 energies: the
        // candidates on the asked side exactly (FP64, as the reference)
        auto rescan = [&](bool scan_hi, bool scan_lo) {
            for (int i = tid; i < n; i += BS) {
                float E;
                if (exact) {
                    E = member_energy(false, A, qr[i], qv[i], pot[i], dcm, scm, inv_d, opz_d);
                } else {
                    float dd, pe;
                    E = staged_energy(qw[i], pot[i], wx, wy, wz, epot, dd, pe);
                }
                const bool ch = scan_hi && E >= hi, cl = scan_lo && E <= lo;
                if (ch || cl) {
                    const float X = exact_energy(A, qr[i], qv[i], pot[i], dcm, inv_d, opz_d);
                    if (ch && X > mx.v) { mx.v = X; mx.i = i; }
                    if (cl && X < mn.v) { mn.v = X; mn.i = i; }
                }
            }
        };
        // The arg-max.  One candidate alone is the exact arg-max (every other
        // member's exact energy is below gmax - bnd, its own at least that),
        // and the sign of its exact energy is known when gmax >= bnd or
        // gmax < -bnd: the usual pass evaluates no FP64 energy.  The warps'
        // candidate counts ride on the barrier the block needs anyway (a
        // thread with two candidates counts as two).
        {
            const unsigned bal = __ballot_sync(SKID_FULL, t1.v >= hi);
            const int first = __shfl_sync(SKID_FULL, t1.i, bal ? __ffs(bal) - 1 : 0);
            const bool two = __any_sync(SKID_FULL, x2.v >= hi);
            if (lane == 0) {
                S.ccnt[w] = __popc(bal) + (two ? 2 : 0);
                S.cidx[w] = first;
            }
            if (bal && lane == __ffs(bal) - 1) {
                S.cr[w] = qr[t1.i];
                S.cv[w] = qv[t1.i];
                S.cw[w] = exact ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : qw[t1.i];
                S.cp[w] = pot[t1.i];
                S.cid[w] = qid[t1.i];
            }
        }
        __syncthreads();
        int ccnt = 0, cidx = 0, kw = 0;
        for (int k = 0; k < BS / 32; ++k) {
            const int c = S.ccnt[k];
            if (c && !ccnt) {
                cidx = S.cidx[k];
                kw = k;
            }
            ccnt += c;
        }
        bool go;
        int ib = cidx;
        if (ccnt == 1 && gmax >= bnd) {
            go = true;
        } else if (ccnt == 1 && gmax < -bnd) {
            go = false;
        } else {
            mx = ArgRed{-FLT_MAX, 0x7fffffff};
            if (t1.i < n && t1.v >= hi && x2.v < hi) {
                mx.v = exact_energy(A, qr[t1.i], qv[t1.i], pot[t1.i], dcm, inv_d, opz_d);
                mx.i = t1.i;
            }
            if (x2.v >= hi) rescan(true, false);
            mx = warp_argmax(mx);
            if (lane == 0) S.smax[w] = mx;
            __syncthreads();
            ArgRed a = S.smax[0];
            for (int k = 1; k < BS / 32; ++k) {
                const ArgRed x = S.smax[k];
                if (x.v > a.v || (x.v == a.v && x.i < a.i)) a = x;
            }
            go = a.v >= 0.0f;   // kd.c:1389-1409: fTotBig starts at -1
            ib = a.i;
            kw = BS / 32;
            if (go && tid == 0) {
                S.cr[kw] = qr[ib];
                S.cv[kw] = qv[ib];
                S.cw[kw] = exact ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : qw[ib];
                S.cp[kw] = pot[ib];
                S.cid[kw] = qid[ib];
            }
            __syncthreads();
        }
        if (A.nounbind || n == 0) go = false;
        if (!go) {
            // the group's most bound member (fTotMin starts at 1), needed
            // only once the removals stop
            mn = ArgRed{FLT_MAX, 0x7fffffff};
            if (b1.i < n && b1.v <= lo && n2.v > lo) {
                mn.v = exact_energy(A, qr[b1.i], qv[b1.i], pot[b1.i], dcm, inv_d, opz_d);
                mn.i = b1.i;
            }
            if (n2.v <= lo) rescan(false, true);
            mn = warp_argmin(mn);
            if (lane == 0) S.smin[w] = mn;
            __syncthreads();
            if (tid == 0) {
                ArgRed b = S.smin[0];
                for (int k = 1; k < BS / 32; ++k) {
                    const ArgRed y = S.smin[k];
                    if (y.v < b.v || (y.v == b.v && y.i < b.i)) b = y;
                }
                S.s_imin = b.v < 1.0f ? b.i : 0;
            }
            break;
        }
        // Remove member ib, swapping the last member into its slot
        // (kd.c:1424-1440): thread 0 updates the FP64 centre while thread 32
        // moves the records, both from records already read.
        const int nn = n - 1;
        if (tid == 0) {
            const float4 r_ib = S.cr[kw], v_ib = S.cv[kw];
            A.grp[S.cid[kw]] = 0;
            ++nrem;
            if (nn == 0) {
                S.d_mass = 0.0;
                for (int d = 3; d < 6; ++d) S.d_cm[d] = 0.0;
            } else {
                double mm = S.d_mass;
                rcm_update(mm, dcm, r_ib, v_ib);
                S.d_mass = mm;
                for (int d = 0; d < 6; ++d) {
                    S.d_cm[d] = dcm[d];
                    S.s_cm[d] = (float)dcm[d];
                }
                if (!exact) {
                    for (int d = 0; d < 3; ++d)
                        S.s_w[d] = (float)((double)A.fShift * dcm[3 + d] + (double)A.fCosmo * dcm[d]);
                    S.s_mW = centre_mag(A, dcm);
                }
                S.s_r = r_ib;
                S.s_eps = v_ib.w;
                S.s_have = 1;
            }
            S.s_n = nn;
        } else if (tid == 32 && nn > 0) {
            qr[ib] = lr; qv[ib] = lv; qid[ib] = lq; pot[ib] = lp;
            qr[nn] = S.cr[kw]; qv[nn] = S.cv[kw]; qid[nn] = S.cid[kw]; pot[nn] = S.cp[kw];
            if (!exact) {
                qw[ib] = lw;
                qw[nn] = S.cw[kw];
            }
        }
        __syncthreads();
        if (nn == 0) break;
    }
    if (tid == 0) {
        double dcm[6];
        for (int d = 0; d < 6; ++d) dcm[d] = S.d_cm[d];
        write_record(A, g, S.s_n, S.d_mass, dcm, qr[S.s_imin], nrem);
    }
    __syncthreads();
}

// ---- the largest groups: one thread-block cluster each ----
//
// One of the largest groups can be shared by the CS blocks of one cluster.
// Block c holds slots [c Q, (c+1) Q) of the members (Q = ceil(n0 / CS)) in
// shared memory: relative position and mass, the staged w = a v + aH r with
// the softening, and the fixed-point potential, so every pass reads on-chip
// memory instead of L2.  A removal takes three cluster barriers:
//   1. each block's FP32 extremes and error-bound terms are gathered from
//      all blocks' shared memory (distributed shared memory) and combined in
//      rank order, so every block holds the same candidate thresholds;
//   2. likewise the blocks' exact arg-max and arg-min (first index on ties)
//      give every block the same decision; each reads the removed member from
//      its owner block and updates its FP64 centre;
//   3. once all have read it, the owner of the freed slot copies the last
//      member into it (swap with the last, kd.c:1435-1440).
// Velocities, positions and ids in global memory are swapped the same way:
// velocities are read only for the exact energies of the few candidates and
// for the removed member.
struct ClusterShared {
    float part[4];          // block FP32 max, min, max dd, max |pe|
    ArgRed pmax, pmin;      // block exact arg-max, arg-min
    double psum[7];         // block FP64 sums: mass, m r, m v
    float pmg;              // block max |a v_j| + |aH r_j|
    int item;
};

template <int BS, int CS>
__device__ void cluster_group(const RemoveArgs &A, int g, BlockShared<BS> &S, ClusterShared &C,
                              float4 *dyn, cg::cluster_group &cl)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int rank = (int)cl.block_rank();
    const int s = A.gstart[g], n0 = A.gcount[g];
    const int Q = (n0 + CS - 1) / CS;
    const int lo = rank * Q, hi = min(lo + Q, n0);
    float4 *s_r = dyn, *s_w = dyn + A.qcap;
    long long *s_p = reinterpret_cast<long long *>(dyn + 2 * A.qcap);
    float4 *qr = A.qr + s, *qv = A.qv + s;
    int *qid = A.qid + s;
    const long long *pot = A.pot + s;
    // the slice into shared memory, its FP64 sums and member magnitudes
    double m = 0.0, c[6] = {0, 0, 0, 0, 0, 0};
    float mg = 0.0f;
    for (int i = lo + tid; i < hi; i += BS) {
        const float4 r = qr[i], v = qv[i];
        s_r[i - lo] = r;
        s_w[i - lo] = make_float4(__fmaf_rn(A.fShift, v.x, A.fCosmo * r.x),
                                  __fmaf_rn(A.fShift, v.y, A.fCosmo * r.y),
                                  __fmaf_rn(A.fShift, v.z, A.fCosmo * r.z), v.w);
        s_p[i - lo] = pot[i];
        m += r.w;
        c[0] += fmul(r.w, r.x); c[1] += fmul(r.w, r.y); c[2] += fmul(r.w, r.z);
        c[3] += fmul(r.w, v.x); c[4] += fmul(r.w, v.y); c[5] += fmul(r.w, v.z);
        mg = fmaxf(mg, fabsf(A.fShift * v.x) + fabsf(A.fCosmo * r.x));
        mg = fmaxf(mg, fabsf(A.fShift * v.y) + fabsf(A.fCosmo * r.y));
        mg = fmaxf(mg, fabsf(A.fShift * v.z) + fabsf(A.fCosmo * r.z));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        m += __shfl_xor_sync(SKID_FULL, m, o);
        for (int d = 0; d < 6; ++d) c[d] += __shfl_xor_sync(SKID_FULL, c[d], o);
    }
    mg = __uint_as_float(__reduce_max_sync(SKID_FULL, __float_as_uint(mg)));
    if (lane == 0) {
        S.part[w][0] = m;
        for (int d = 0; d < 6; ++d) S.part[w][1 + d] = c[d];
        S.ext[w][0] = mg;
    }
    __syncthreads();
    if (tid == 0) {
        double t[7] = {0, 0, 0, 0, 0, 0, 0};
        float tm = 0.0f;
        for (int k = 0; k < BS / 32; ++k) {
            for (int d = 0; d < 7; ++d) t[d] += S.part[k][d];
            tm = fmaxf(tm, S.ext[k][0]);
        }
        for (int d = 0; d < 7; ++d) C.psum[d] = t[d];
        C.pmg = tm;
    }
    cl.sync();
    if (tid == 0) {
        // every block combines the partials in rank order: the same values
        double t[7] = {0, 0, 0, 0, 0, 0, 0};
        float tm = 0.0f;
        for (int b = 0; b < CS; ++b) {
            const ClusterShared *rc = cl.map_shared_rank(&C, b);
            for (int d = 0; d < 7; ++d) t[d] += rc->psum[d];
            tm = fmaxf(tm, rc->pmg);
        }
        S.d_mass = t[0];
        for (int d = 0; d < 6; ++d) {
            S.d_cm[d] = t[1 + d] / t[0];
            S.s_cm[d] = (float)S.d_cm[d];
        }
        for (int d = 0; d < 3; ++d)
            S.s_w[d] = (float)((double)A.fShift * S.d_cm[3 + d] + (double)A.fCosmo * S.d_cm[d]);
        S.s_mg = tm * 1.0000002f;
        S.s_mW = centre_mag(A, S.d_cm);
        S.s_n = n0;
        S.s_have = 0;
        S.s_go = 1;
    }
    cl.sync();   // every block has read the sums before any overwrites them
    int nrem = 0;
    const double opz_d = 1.0 + (double)A.z, inv_d = 1.0 / (double)A.scale;
    const float epot = A.inv_scale * A.opz;
    for (;;) {
        const int n = S.s_n;
        const bool sub = S.s_have != 0 && A.subpot;
        const float4 rs = S.s_r;
        const float es = S.s_eps;
        double dcm[6];
        for (int d = 0; d < 6; ++d) dcm[d] = S.d_cm[d];
        const float wx = S.s_w[0], wy = S.s_w[1], wz = S.s_w[2];
        const float gms = fmul(A.G, rs.w) * A.scale;
        ArgRed mx{-FLT_MAX, 0x7fffffff}, mn{FLT_MAX, 0x7fffffff};
        ArgRed mx2 = mx, mn2 = mn;
        float ddmx = 0.0f, pemx = 0.0f;
        const int e = min(hi, n);
        for (int i = lo + tid; i < e; i += BS) {
            const float4 r = s_r[i - lo], wv = s_w[i - lo];
            long long p = s_p[i - lo];
            if (sub) {
                // kdSubPot (grav.c:44-59): the term the potentials added
                const float d2 = d2of(fsub(rs.x, r.x), fsub(rs.y, r.y), fsub(rs.z, r.z));
                p -= fx(fmul(gms, pair_dir(d2, fadd(es, wv.w), A.plummer)), 1.0f);
                s_p[i - lo] = p;
            }
            const float dx = wv.x - wx, dy = wv.y - wy, dz = wv.z - wz;
            const float dd = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
            const float pe = ll2f_fast(p) * epot;
            const float E = 0.5f * dd - pe;
            keep_top2(mx, mx2, E, i);
            keep_bot2(mn, mn2, E, i);
            ddmx = fmaxf(ddmx, dd);
            pemx = fmaxf(pemx, fabsf(pe));
        }
        // 1. the FP32 extremes and bound terms over the whole group
        {
            float a0 = mx.v, a1 = mn.v, a2 = ddmx, a3 = pemx;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                a0 = fmaxf(a0, __shfl_xor_sync(SKID_FULL, a0, o));
                a1 = fminf(a1, __shfl_xor_sync(SKID_FULL, a1, o));
                a2 = fmaxf(a2, __shfl_xor_sync(SKID_FULL, a2, o));
                a3 = fmaxf(a3, __shfl_xor_sync(SKID_FULL, a3, o));
            }
            if (lane == 0) {
                S.ext[w][0] = a0;
                S.ext[w][1] = a1;
                S.ext[w][2] = a2;
                S.ext[w][3] = a3;
            }
            __syncthreads();
            if (tid == 0) {
                float b0 = -FLT_MAX, b1 = FLT_MAX, b2 = 0.0f, b3 = 0.0f;
                for (int k = 0; k < BS / 32; ++k) {
                    b0 = fmaxf(b0, S.ext[k][0]);
                    b1 = fminf(b1, S.ext[k][1]);
                    b2 = fmaxf(b2, S.ext[k][2]);
                    b3 = fmaxf(b3, S.ext[k][3]);
                }
                C.part[0] = b0;
                C.part[1] = b1;
                C.part[2] = b2;
                C.part[3] = b3;
            }
        }
        cl.sync();
        if (tid < CS) {
            // thread b fetches block b's partials from its shared memory
            const ClusterShared *rc = cl.map_shared_rank(&C, tid);
            for (int d = 0; d < 4; ++d) S.gpart[tid][d] = rc->part[d];
        }
        __syncthreads();
        float gmax = -FLT_MAX, gmin = FLT_MAX, gdd = 0.0f, gpe = 0.0f;
        for (int b = 0; b < CS; ++b) {
            gmax = fmaxf(gmax, S.gpart[b][0]);
            gmin = fminf(gmin, S.gpart[b][1]);
            gdd = fmaxf(gdd, S.gpart[b][2]);
            gpe = fmaxf(gpe, S.gpart[b][3]);
        }
        // the staged path's bound (block_group, groups above 1024 members)
        const float Cm = S.s_mg + S.s_mW;
        const float bound =
            1.9073486e-06f * (Cm * (1.7320509f * sqrtf(gdd) + 3.0f * Cm) + 1.5f * gdd + 2.0f * gpe) +
            1e-30f;
        const float hiE = gmax - 2.0f * bound, loE = gmin + 2.0f * bound;
        const ArgRed t1 = mx, b1 = mn;
        mx = ArgRed{-FLT_MAX, 0x7fffffff};
        mn = ArgRed{FLT_MAX, 0x7fffffff};
        if (t1.i < e && t1.v >= hiE && mx2.v < hiE) {
            mx.v = exact_energy(A, s_r[t1.i - lo], qv[t1.i], s_p[t1.i - lo], dcm, inv_d, opz_d);
            mx.i = t1.i;
        }
        if (b1.i < e && b1.v <= loE && mn2.v > loE) {
            mn.v = exact_energy(A, s_r[b1.i - lo], qv[b1.i], s_p[b1.i - lo], dcm, inv_d, opz_d);
            mn.i = b1.i;
        }
        const bool scan_hi = mx2.v >= hiE, scan_lo = mn2.v <= loE;
        if (scan_hi || scan_lo) {
            for (int i = lo + tid; i < e; i += BS) {
                const float4 wv = s_w[i - lo];
                const long long p = s_p[i - lo];
                const float dx = wv.x - wx, dy = wv.y - wy, dz = wv.z - wz;
                const float E =
                    0.5f * __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx)) - ll2f_fast(p) * epot;
                const bool ch = scan_hi && E >= hiE, clo = scan_lo && E <= loE;
                if (ch || clo) {
                    const float X = exact_energy(A, s_r[i - lo], qv[i], p, dcm, inv_d, opz_d);
                    if (ch && X > mx.v) { mx.v = X; mx.i = i; }
                    if (clo && X < mn.v) { mn.v = X; mn.i = i; }
                }
            }
        }
        // 2. the exact arg-max and arg-min over the whole group
        mx = warp_argmax(mx);
        mn = warp_argmin(mn);
        if (lane == 0) { S.smax[w] = mx; S.smin[w] = mn; }
        __syncthreads();
        if (tid == 0) {
            ArgRed a = S.smax[0], b = S.smin[0];
            for (int k = 1; k < BS / 32; ++k) {
                const ArgRed x = S.smax[k], y = S.smin[k];
                if (x.v > a.v || (x.v == a.v && x.i < a.i)) a = x;
                if (y.v < b.v || (y.v == b.v && y.i < b.i)) b = y;
            }
            C.pmax = a;
            C.pmin = b;
        }
        cl.sync();
        if (tid < CS) {
            const ClusterShared *rc = cl.map_shared_rank(&C, tid);
            S.gmx[tid] = rc->pmax;
            S.gmn[tid] = rc->pmin;
        }
        __syncthreads();
        if (tid == 0) {
            ArgRed a = S.gmx[0], b = S.gmn[0];
            for (int k = 1; k < CS; ++k) {
                const ArgRed x = S.gmx[k], y = S.gmn[k];
                if (x.v > a.v || (x.v == a.v && x.i < a.i)) a = x;
                if (y.v < b.v || (y.v == b.v && y.i < b.i)) b = y;
            }
            // kd.c:1389-1409: fTotBig starts at -1, fTotMin at 1
            S.s_imin = b.v < 1.0f ? b.i : 0;
            if (!(a.v >= 0.0f) || A.nounbind || n == 0) {
                S.s_go = 0;
            } else {
                const int ib = a.i;
                const int ob = ib / Q;
                const float4 r = cl.map_shared_rank(s_r, ob)[ib - ob * Q];
                const float4 wv = cl.map_shared_rank(s_w, ob)[ib - ob * Q];
                const float4 v = qv[ib];
                if (rank == 0) A.grp[qid[ib]] = 0;
                ++nrem;
                const int nn = n - 1;
                if (nn == 0) {
                    S.d_mass = 0.0;
                    for (int d = 3; d < 6; ++d) S.d_cm[d] = 0.0;
                    S.s_go = 0;
                } else {
                    double mm = S.d_mass;
                    for (int d = 0; d < 6; ++d) dcm[d] = S.d_cm[d];
                    rcm_update(mm, dcm, r, v);
                    S.d_mass = mm;
                    for (int d = 0; d < 6; ++d) {
                        S.d_cm[d] = dcm[d];
                        S.s_cm[d] = (float)dcm[d];
                    }
                    for (int d = 0; d < 3; ++d)
                        S.s_w[d] = (float)((double)A.fShift * dcm[3 + d] + (double)A.fCosmo * dcm[d]);
                    S.s_mW = centre_mag(A, dcm);
                    S.s_r = r;
                    S.s_eps = wv.w;
                    S.s_have = 1;
                }
                S.s_n = nn;
                S.s_item = ib;
            }
        }
        // 3. every block has read the removed member (and rank 0 its id)
        // before its slot is overwritten
        cl.sync();
        if (tid == 0 && S.s_go) {
            const int ib = S.s_item;
            const int nn = S.s_n;
            if (ib / Q == rank && ib != nn) {
                const int on = nn / Q;
                s_r[ib - lo] = cl.map_shared_rank(s_r, on)[nn - on * Q];
                s_w[ib - lo] = cl.map_shared_rank(s_w, on)[nn - on * Q];
                s_p[ib - lo] = cl.map_shared_rank(s_p, on)[nn - on * Q];
                const float4 rl = qr[nn], vl = qv[nn], rb = qr[ib], vb = qv[ib];
                const int il = qid[nn], ir = qid[ib];
                qr[ib] = rl; qv[ib] = vl; qid[ib] = il;
                qr[nn] = rb; qv[nn] = vb; qid[nn] = ir;
            }
        }
        __syncthreads();
        if (!S.s_go) break;
    }
    if (rank == 0 && tid == 0) {
        double dcm[6];
        for (int d = 0; d < 6; ++d) dcm[d] = S.d_cm[d];
        write_record(A, g, S.s_n, S.d_mass, dcm, qr[S.s_imin], nrem);
    }
    cl.sync();   // no block leaves while another may still read its shared memory
}

// Persistent removal: queue items [0, nbig) are large groups (one block
// each), then chunks of BS/32 small groups (one warp each), all largest
// first.  With A.single > 0 one block processes just that group.
template <int BS, int CS>
__global__ void __launch_bounds__(BS) remove_kernel(RemoveArgs A)
{
    __shared__ BlockShared<BS> S;
    __shared__ int s_item;
    constexpr int W = BS / 32;
    if (A.single > 0) {
        block_group<BS>(A, A.single, S);
        return;
    }
    int first = 0;
    if constexpr (CS > 1) {
        // launched as clusters of CS blocks: the largest groups first, one
        // cluster each, then every block goes on alone
        __shared__ ClusterShared C;
        extern __shared__ float4 dyn[];
        cg::cluster_group cl = cg::this_cluster();
        const int nclu = *A.d_ccnt;
        for (;;) {
            if (cl.block_rank() == 0 && threadIdx.x == 0) C.item = atomicAdd(A.d_cqueue, 1);
            cl.sync();
            const int item = cl.map_shared_rank(&C, 0)->item;
            cl.sync();
            if (item >= nclu) break;
            cluster_group<BS, CS>(A, (int)A.order[item], S, C, dyn, cl);
        }
        first = nclu;
    }
    const int nvalid = A.d_cnt[0], nbig = A.d_cnt[1] > first ? A.d_cnt[1] : first;
    const int nb = nbig - first;
    const int nitems = nb + (nvalid - nbig + W - 1) / W;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(A.d_queue, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= nitems) break;
        if (item < nb) {
            block_group<BS>(A, (int)A.order[first + item], S);
        } else {
            int k = nbig + (item - nb) * W + (threadIdx.x >> 5);
            if (k < nvalid) warp_group(A, (int)A.order[k]);
        }
    }
}

template <int BS>
cudaError_t launch_remove(const RemoveArgs &A, int blocks, cudaStream_t st)
{
    remove_kernel<BS, 1><<<blocks, BS, 0, st>>>(A); note_launch();
    return cudaGetLastError();
}

// Cluster launch: as many clusters of CS blocks as fit at once, each block
// with A.qcap members' worth of dynamic shared memory.
template <int BS, int CS>
cudaError_t launch_remove_clusters(const RemoveArgs &A, cudaStream_t st)
{
    const size_t smem = (size_t)A.qcap * (2 * sizeof(float4) + sizeof(long long));
    cudaError_t e = cudaFuncSetAttribute(remove_kernel<BS, CS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(BS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(CS, 1, 1);
    int nclusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&nclusters, remove_kernel<BS, CS>, &cfg))) return e;
    if (nclusters < 1) return cudaErrorInvalidConfiguration;
    cfg.gridDim = dim3(CS * nclusters, 1, 1);
    e = cudaLaunchKernelEx(&cfg, remove_kernel<BS, CS>, A);
    note_launch();
    return e ? e : cudaGetLastError();
}

// cs: 1 (no clusters), 4 or 8
cudaError_t remove_launch(const RemoveArgs &A, int bs, int cs, int blocks, cudaStream_t st)
{
    if (cs == 4 || cs == 8) {
        switch (bs) {
        case 512: return cs == 4 ? launch_remove_clusters<512, 4>(A, st) : launch_remove_clusters<512, 8>(A, st);
        case 1024: return cs == 4 ? launch_remove_clusters<1024, 4>(A, st) : launch_remove_clusters<1024, 8>(A, st);
        default: return cs == 4 ? launch_remove_clusters<256, 4>(A, st) : launch_remove_clusters<256, 8>(A, st);
        }
    }
    switch (bs) {
    case 128: return launch_remove<128>(A, blocks, st);
    case 512: return launch_remove<512>(A, blocks, st);
    case 1024: return launch_remove<1024>(A, blocks, st);
    default: return launch_remove<256>(A, blocks, st);
    }
}

int remove_blocks(int bs)
{
    int perSM = 0;
    switch (bs) {
    case 128: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, remove_kernel<128, 1>, 128, 0); break;
    case 512: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, remove_kernel<512, 1>, 512, 0); break;
    case 1024: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, remove_kernel<1024, 1>, 1024, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, remove_kernel<256, 1>, 256, 0); break;
    }
    return num_sms() * (perSM > 0 ? perSM : 1);
}

}  // namespace

// Candidate removal schedules (tw, BS) for the autotuner.
static const int kTW[] = {0, 32, 128, 256, 512, 1024};
static const int kBS[] = {256, 512, 1024};

cudaError_t unbind_run(GroupState &G, const int *gof, int nslots, const float4 *pos4,
                       const float4 *vel4, Tree &ut, const UnbindParams &P, int *grp,
                       int *d_unbound, SortScratch &ss, UnbindScratch &U, cudaStream_t st)
{
    cudaError_t e;
    int ng = G.nGroup;
    if ((e = dalloc(U.qr, nslots)) || (e = dalloc(U.qv, nslots)) || (e = dalloc(U.qw, nslots)) ||
        (e = dalloc(U.qid, nslots)) ||
        (e = dalloc(U.pot, nslots)) || (e = dalloc(U.scnt, ng)) || (e = dalloc(U.soff, ng + 1)) ||
        (e = dalloc(U.nt, ng)) || (e = dalloc(U.toff, ng + 1)) || (e = dalloc(U.cnt, 16)) ||
        (e = dalloc(U.order, ng)))
        return e;
    float3 hP = make_float3((float)(0.5 * (double)P.period.x), (float)(0.5 * (double)P.period.y),
                            (float)(0.5 * (double)P.period.z));
    auto prep = [&]() -> cudaError_t {
        prep_members<<<grid_for(nslots), 256, 0, st>>>(G.members.p, gof, nslots, pos4, vel4, G.rec.p,
                                                       hP, U.qr.p, U.qv.p); note_launch();
        return cudaMemcpyAsync(U.qid.p, G.members.p, nslots * sizeof(int), cudaMemcpyDeviceToDevice, st);
    };
    if ((e = prep())) return e;
    // scoop lists
    float fBall2 = P.fScoop * P.fScoop;
    float3 hL = make_float3(0.5f * P.period.x, 0.5f * P.period.y, 0.5f * P.period.z);
    scoop_kernel<<<grid_for(ng), 256, 0, st>>>(ut.view(), U.usoft.p, G.rec.p, G.count.p, ng, P.nmax,
                                              fBall2, P.period, hL, P.per, 0, U.scnt.p, nullptr,
                                              nullptr, nullptr); note_launch();
    if ((e = scan_exclusive(U.scnt.p, U.soff.p, ng, U.cnt.p, ss, st))) return e;
    int nscoop = 0;
    if ((e = cudaMemcpyAsync(&nscoop, U.cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    if ((e = dalloc(U.slist, nscoop > 0 ? nscoop : 1)) || (e = dalloc(U.ssoft, nscoop > 0 ? nscoop : 1)))
        return e;
    if (nscoop > 0)
        scoop_kernel<<<grid_for(ng), 256, 0, st>>>(ut.view(), U.usoft.p, G.rec.p, G.count.p, ng,
                                                  P.nmax, fBall2, P.period, hL, P.per, 1, U.scnt.p,
                                                  U.soff.p, U.slist.p, U.ssoft.p); note_launch();
    // groups by descending size
    if ((e = dalloc(ss.k0, ng)) || (e = dalloc(ss.v0, ng)) || (e = dalloc(ss.k1, ng)) ||
        (e = dalloc(ss.v1, ng)))
        return e;
    sched_keys<<<grid_for(ng), 256, 0, st>>>(G.count.p, ng, P.nmax, ss.k0.p, ss.v0.p); note_launch();
    if ((e = radix_sort(ss, ng, 32, st))) return e;
    if ((e = cudaMemcpyAsync(U.order.p, ss.v0.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st)))
        return e;
    if ((e = cudaMemsetAsync(U.cnt.p + 2, 0, 2 * sizeof(int), st))) return e;
    sched_counts<<<grid_for(ng), 256, 0, st>>>(G.count.p, ng, P.nmax, 1 << 30, U.cnt.p + 2); note_launch();
    // potential items, largest groups first
    pot_nitems<<<grid_for(ng), 256, 0, st>>>(U.order.p, U.cnt.p + 2, G.count.p, ng, U.nt.p); note_launch();
    if ((e = scan_exclusive(U.nt.p, U.toff.p, ng, U.cnt.p + 1, ss, st))) return e;
    // clustered groups: the largest ones above clu_min members, at most as
    // many as keep half the SMs busy with clusters of 4 blocks; and the
    // largest group's size, which sizes the blocks' shared-memory slices
    const int clu_min = P.clu_min > P.tw && P.clu_min > 1024 ? P.clu_min : 0;
    const int clu_kmax = num_sms() / 8 > 1 ? num_sms() / 8 : 1;
    if ((e = cudaMemsetAsync(U.cnt.p + 8, 0, 4 * sizeof(int), st))) return e;
    if (clu_min > 0) {
        cluster_groups<<<1, 32, 0, st>>>(U.order.p, U.cnt.p + 2, G.count.p, clu_min, clu_kmax,
                                         U.cnt.p + 9); note_launch();
    }
    int hc[11] = {0};
    if ((e = cudaMemcpyAsync(hc, U.cnt.p + 1, 11 * sizeof(int), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    const int nitems = hc[0], nvalid = hc[1], nclu = hc[8], nlargest = hc[10];
    // cluster size: 4 blocks while a quarter of the largest group fits in
    // about 200 KB of shared memory (40 B per member), else 8, else none
    int cs = 1, qcap = 0;
    if (clu_min > 0 && nclu > 0) {
        const int per = (int)(2 * sizeof(float4) + sizeof(long long));
        const int q4 = (nlargest + 3) / 4, q8 = (nlargest + 7) / 8;
        if ((size_t)q4 * per <= 200u * 1024u) { cs = 4; qcap = q4; }
        else if ((size_t)q8 * per <= 200u * 1024u) { cs = 8; qcap = q8; }
    }
    if ((e = dalloc(U.items, nitems > 0 ? nitems : 1))) return e;
    if (nitems > 0)
        pot_fill<<<grid_for(nvalid), 256, 0, st>>>(U.order.p, U.cnt.p + 2, G.count.p, U.toff.p,
                                                   U.items.p); note_launch();

    RemoveArgs A;
    A.gstart = G.start.p;
    A.gcount = G.count.p;
    A.ng = ng;
    A.nmax = P.nmax;
    A.qr = U.qr.p;
    A.qv = U.qv.p;
    A.qw = U.qw.p;
    A.qid = U.qid.p;
    A.pot = U.pot.p;
    A.rec = G.rec.p;
    A.grp = grp;
    A.d_unbound = d_unbound;
    A.G = P.G;
    A.fShift = P.a;
    A.fCosmo = P.aH;
    A.opz = P.opz;
    A.z = P.z;
    A.scale = P.scale;
    A.inv_scale = 1.0f / P.scale;
    A.hP = hP;
    A.plummer = P.plummer;
    A.subpot = P.subpot;
    A.nounbind = P.nounbind;
    A.order = U.order.p;
    A.d_cnt = U.cnt.p + 4;
    A.d_queue = U.cnt.p + 6;
    A.d_ccnt = U.cnt.p + 9;
    A.d_cqueue = U.cnt.p + 10;
    A.qcap = qcap;
    A.single = 0;

    const int potBlocks = nitems < num_sms() * 32 ? (nitems > 0 ? nitems : 1) : num_sms() * 32;
    auto potentials = [&]() -> cudaError_t {
        cudaError_t e2 = cudaMemsetAsync(U.pot.p, 0, nslots * sizeof(long long), st);
        if (e2 || nitems <= 0) return e2;
        pot_sym_kernel<<<potBlocks, POT_THREADS, 0, st>>>(U.items.p, U.cnt.p + 1, -1, G.start.p, G.count.p,
                                                       U.qr.p, U.qv.p, U.soff.p, U.scnt.p, U.slist.p,
                                                       U.ssoft.p, P.G, P.plummer, P.scale, U.pot.p); note_launch();
        return cudaGetLastError();
    };
    auto removal = [&](int tw, int bs, int ucs) -> cudaError_t {
        cudaError_t e2;
        if ((e2 = cudaMemsetAsync(U.cnt.p + 4, 0, 3 * sizeof(int), st))) return e2;
        if ((e2 = cudaMemsetAsync(U.cnt.p + 10, 0, sizeof(int), st))) return e2;
        sched_counts<<<grid_for(ng), 256, 0, st>>>(G.count.p, ng, P.nmax, tw, U.cnt.p + 4); note_launch();
        if ((e2 = cudaMemsetAsync(d_unbound, 0, sizeof(int), st))) return e2;
        if (nvalid <= 0) return cudaSuccess;
        return remove_launch(A, bs, bs >= 256 ? ucs : 1, remove_blocks(bs), st);
    };

    if (P.per_group) {
        // the reference's serial loop on the GPU: two launches per group
        std::vector<uint32_t> order(ng);
        std::vector<int> ioff(ng + 1);
        if ((e = cudaMemcpyAsync(order.data(), U.order.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaMemcpyAsync(ioff.data(), U.toff.p, ng * sizeof(int), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st)))
            return e;
        ioff[nvalid] = nitems;
        if ((e = cudaMemsetAsync(U.pot.p, 0, nslots * sizeof(long long), st))) return e;
        if ((e = cudaMemsetAsync(d_unbound, 0, sizeof(int), st))) return e;
        for (int k = 0; k < nvalid; ++k) {
            int cnt = ioff[k + 1] - ioff[k];
            pot_sym_kernel<<<cnt < num_sms() * 32 ? cnt : num_sms() * 32, POT_THREADS, 0, st>>>(
                U.items.p + ioff[k], nullptr, cnt, G.start.p, G.count.p, U.qr.p, U.qv.p, U.soff.p,
                U.scnt.p, U.slist.p, U.ssoft.p, P.G, P.plummer, P.scale, U.pot.p); note_launch();
            RemoveArgs A1 = A;
            A1.single = (int)order[k];
            if ((e = remove_launch(A1, 256, 1, 1, st))) return e;
        }
        return cudaGetLastError();
    }

    cudaEvent_t t0 = nullptr, t1 = nullptr, t2 = nullptr;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventCreate(&t2);
    cudaEventRecord(t0, st);
    if ((e = potentials())) return e;
    cudaEventRecord(t1, st);
    int tw = P.tw, bs = P.bs;
    if ((tw < 0 || bs < 0) && U.tuned_bs > 0) {
        if (tw < 0) tw = U.tuned_tw;
        if (bs < 0) bs = U.tuned_bs;
    }
    if (tw < 0 || bs < 0) {
        // autotune: time every candidate removal schedule on these groups,
        // restoring the inputs between runs, then keep the fastest
        if ((e = dalloc(U.pot_save, nslots)) || (e = dalloc(U.rec_save, ng)) ||
            (e = dalloc(U.grp_save, P.n > 0 ? P.n : 1)))
            return e;
        if ((e = cudaMemcpyAsync(U.pot_save.p, U.pot.p, nslots * sizeof(long long), cudaMemcpyDeviceToDevice, st)) ||
            (e = cudaMemcpyAsync(U.rec_save.p, G.rec.p, ng * sizeof(skid_group), cudaMemcpyDeviceToDevice, st)) ||
            (e = cudaMemcpyAsync(U.grp_save.p, grp, P.n * sizeof(int), cudaMemcpyDeviceToDevice, st)))
            return e;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = FLT_MAX;
        int btw = 32, bbs = 256;
        for (int a : kTW) {
            if (P.tw >= 0 && a != P.tw) continue;
            for (int b : kBS) {
                if (P.bs >= 0 && b != P.bs) continue;
                if ((e = cudaMemcpyAsync(U.pot.p, U.pot_save.p, nslots * sizeof(long long), cudaMemcpyDeviceToDevice, st)) ||
                    (e = cudaMemcpyAsync(G.rec.p, U.rec_save.p, ng * sizeof(skid_group), cudaMemcpyDeviceToDevice, st)) ||
                    (e = cudaMemcpyAsync(grp, U.grp_save.p, P.n * sizeof(int), cudaMemcpyDeviceToDevice, st)) ||
                    (e = prep()))
                    break;
                cudaEventRecord(e0, st);
                if ((e = removal(a, b, 1))) break;
                cudaEventRecord(e1, st);
                if ((e = cudaEventSynchronize(e1))) break;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                U.tune_ms[U.ntune < 32 ? U.ntune : 31] = ms;
                ++U.ntune;
                U.ntune_now = 1;
                if (ms < best) { best = ms; btw = a; bbs = b; }
            }
            if (e) break;
        }
        // then the best schedule with the largest groups on thread-block
        // clusters, kept only if it is faster
        int bcs = 1;
        if (!e && cs > 1 && bbs >= 256) {
            if (!(e = cudaMemcpyAsync(U.pot.p, U.pot_save.p, nslots * sizeof(long long), cudaMemcpyDeviceToDevice, st)) &&
                !(e = cudaMemcpyAsync(G.rec.p, U.rec_save.p, ng * sizeof(skid_group), cudaMemcpyDeviceToDevice, st)) &&
                !(e = cudaMemcpyAsync(grp, U.grp_save.p, P.n * sizeof(int), cudaMemcpyDeviceToDevice, st)) &&
                !(e = prep())) {
                cudaEventRecord(e0, st);
                e = removal(btw, bbs, cs);
                cudaEventRecord(e1, st);
                if (!e) e = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (!e) cudaEventElapsedTime(&ms, e0, e1);
                U.tune_ms[U.ntune < 32 ? U.ntune : 31] = ms;
                ++U.ntune;
                if (!e && ms < best) bcs = cs;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e) return e;
        U.tuned_tw = btw;
        U.tuned_bs = bbs;
        U.tuned_cs = bcs > 1 ? 1 : 0;
        tw = btw;
        bs = bbs;
        if ((e = cudaMemcpyAsync(U.pot.p, U.pot_save.p, nslots * sizeof(long long), cudaMemcpyDeviceToDevice, st)) ||
            (e = cudaMemcpyAsync(G.rec.p, U.rec_save.p, ng * sizeof(skid_group), cudaMemcpyDeviceToDevice, st)) ||
            (e = cudaMemcpyAsync(grp, U.grp_save.p, P.n * sizeof(int), cudaMemcpyDeviceToDevice, st)) ||
            (e = prep()))
            return e;
    }
    // clusters: as the tuner chose for a tuned schedule; with a fixed one,
    // whenever there are groups for them and the caller set the threshold
    const bool tuned_sched = P.tw < 0 || P.bs < 0;
    const int ucs = cs > 1 && (tuned_sched ? U.tuned_cs == 1 : !P.clu_auto) ? cs : 1;
    U.used_tw = tw;
    U.used_bs = bs;
    U.used_cs = ucs;
    U.used_nclu = ucs > 1 ? nclu : 0;
    if (U.ntune) cudaEventRecord(t1, st);   // tuning ran in between: time the final removal only
    e = removal(tw, bs, ucs);
    cudaEventRecord(t2, st);
    if (!e) e = cudaEventSynchronize(t2);
    float a = 0.0f, b = 0.0f;
    if (!e && !U.ntune_now) cudaEventElapsedTime(&a, t0, t1);
    if (!e) cudaEventElapsedTime(&b, t1, t2);
    if (!U.ntune_now) U.pot_ms = a;
    U.remove_ms = b;
    U.ntune_now = 0;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaEventDestroy(t2);
    return e;
}

}  // namespace skid

// ---- numerics check of the pair factor ----

namespace {

__global__ void pair_factor_kernel(const float *__restrict__ d2, const float *__restrict__ twoh, int n,
                                   int plummer, int mode, float *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float v = __int_as_float(0x7fc00000);   // NaN: the float-float form declined
        if (mode == SKID_PAIR_FP64) v = skid::ref_dir_fp64(d2[i], twoh[i], plummer);
        else if (mode == SKID_PAIR_SPLINE_FF) skid::ref_spline_ff(d2[i], twoh[i], v);
        else v = skid::pair_dir(d2[i], twoh[i], plummer);
        out[i] = v;
    }
}

}  // namespace

extern "C" int skid_pair_factor(int n, const float *d2, const float *twoh, int plummer, int mode,
                                float *out)
{
    if (n < 0 || (n > 0 && (!d2 || !twoh || !out))) return SKID_EINVAL;
    if (mode != SKID_PAIR_USED && mode != SKID_PAIR_FP64 && mode != SKID_PAIR_SPLINE_FF)
        return SKID_EINVAL;
    if (n == 0) return 0;
    float *dv = nullptr;
    const size_t bytes = (size_t)n * sizeof(float);
    {
        std::lock_guard<std::recursive_mutex> lk(skid::device_mutex());
        if (cudaMalloc((void **)&dv, 3 * bytes)) {
            cudaGetLastError();
            return SKID_ENOMEM;
        }
    }
    cudaError_t e = cudaMemcpy(dv, d2, bytes, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dv + n, twoh, bytes, cudaMemcpyHostToDevice);
    if (!e) {
        const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, 65536);
        pair_factor_kernel<<<blocks, 256>>>(dv, dv + n, n, plummer, mode, dv + 2 * (size_t)n);
        skid::note_launch();
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(out, dv + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    {
        std::lock_guard<std::recursive_mutex> lk(skid::device_mutex());
        cudaFree(dv);
    }
    if (e) {
        cudaGetLastError();
        return SKID_ECUDA;
    }
    return 0;
}
