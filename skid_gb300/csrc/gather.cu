// Gather kernels over the scatterer tree.
//
// density_gather: the reference scatters each pair (i, j in NN(i)) to both
// ends (smooth1.c:248-263).  Here each particle gathers both halves itself:
//   rho_i = sum_j 1/2 m_j W(d2(i->j), b_i) [d2 < b_i]     (its own neighbours)
//         + sum_k 1/2 m_k W(d2(k->i), b_k) [d2 < b_k]     (balls that hold it)
// with W the M4 spline of h^2 = b/4.  Each distance is taken in the frame the
// reference uses for that half (the query of the ball).  Deterministic order,
// Kahan-compensated FP32 sums.
//
// field_move: the move step.  The reference has every live scatterer copy
// gather the active movers inside its ball and add m/(pi h^5) F(q)(x_c - y)
// to them (smAccDensity/smBallGather, smooth1.c:338-508), then moves each
// mover by fStep along -a/|a| (kdMoveParticles, kd.c:702-732).  Here each
// mover walks the scatterer tree (ball boxes) and sums the copies whose ball
// holds it, then moves itself in the same kernel; a copy is the scatterer's
// periodic image nearest the mover, x_c = fl(x + sL), and must be live.  The
// warp marks which scatterers it touched (for the density floor of the cut,
// smooth1.c:460-461).
#include <cfloat>

#include "internal.h"

namespace skid {

namespace {

constexpr int G_WARPS = 4;

// Field kernel build tunables: unroll of the candidate test loop, and the
// minimum resident blocks per SM passed to __launch_bounds__ (caps registers).
#ifndef SKID_FIELD_UNROLL
#define SKID_FIELD_UNROLL 4
#endif
#ifndef SKID_FIELD_MINB
#define SKID_FIELD_MINB 12
#endif
constexpr int FIELD_UNROLL = SKID_FIELD_UNROLL;
// Warps a split one-mover-per-warp step aims for (at most FIELD_SPLIT_CAP).
constexpr int FIELD_SPLIT_ITEMS = 8192;
static_assert(FIELD_SPLIT_ITEMS <= FIELD_SPLIT_CAP, "split buffers too small");

__device__ __forceinline__ float w_m4(float r2)
{
    float q = sqrtf(r2);
    float rs = 2.0f - q;
    return r2 < 1.0f ? 1.0f - 0.75f * rs * r2 : 0.25f * rs * rs * rs;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ float shifted(float x, int s, float L)
{
    return s == 0 ? x : (s < 0 ? fsub(x, L) : fadd(x, L));
}

// One warp per leaf of queries.  The walk descends a node while some lane's
// ball reaches its box or some ball below may hold the lane (box distance
// below max(b_i, max ball2 below)); the last 2^subShift leaves of a subtree
// are tested one per lane against the query leaf's box.  At a visited leaf,
// lane j keeps candidate j if its distance to the query box is below
// max(its ball, the largest query ball) -- the only candidates that can
// enter either half -- and the survivors, compacted in order, are summed.
__global__ void __launch_bounds__(G_WARPS * 32)
density_kernel(TreeView t, const float *__restrict__ ball2, float3 L, float3 hL, bool per,
               int subShift, float *__restrict__ rho, int *work)
{
    __shared__ float4 cpos[G_WARPS][SKID_LEAF];
    __shared__ float4 caux[G_WARPS][SKID_LEAF];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int rootLo = t.leafBase >> subShift;
    for (;;) {
        int leaf = 0;
        if (lane == 0) leaf = atomicAdd(work, 1);
        leaf = __shfl_sync(SKID_FULL, leaf, 0);
        if (leaf >= t.nLeaf) break;
        int base = leaf * SKID_LEAF;
        int qi = base + lane;
        bool valid = qi < t.n;
        float4 qp = t.pos[valid ? qi : base];
        float3 q = make_float3(qp.x, qp.y, qp.z);
        float bi = ball2[valid ? qi : base];
        float ih2i = 4.0f / bi;
        float fni = 0.5f * (float)M_1_PI * sqrtf(ih2i) * ih2i;
        // the query leaf's box (its points) and largest ball
        const float4 qlo = t.lo[t.leafBase + leaf], qhi = t.hi[t.leafBase + leaf];
        float s = 0.0f, c = 0.0f;
        int cp = 1;
        for (;;) {
            if (cp >= rootLo) {
                const int first = cp << subShift;
                bool pass = false;
                if (lane < (1 << subShift)) {
                    float4 bl = t.lo[first + lane], bh = t.hi[first + lane];
                    pass = boxbox_lb(qlo, qhi, bl, bh, L, per) < fmaxf(qlo.w, bl.w);
                }
                for (unsigned lm = __ballot_sync(SKID_FULL, pass); lm; lm &= lm - 1) {
                    const int node = first + __ffs(lm) - 1;
                    const int lf = node - t.leafBase;
                    if (lf >= t.nLeaf) break;
                    float4 blo = t.lo[node], bhi = t.hi[node];
                    bool want = box_lb(q, blo, bhi, L, per) < fmaxf(bi, blo.w);
                    if (!__any_sync(SKID_FULL, want)) continue;
                    int cb = lf * SKID_LEAF;
                    int cnt = min(SKID_LEAF, t.n - cb);
                    bool rel = false;
                    float4 cj4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    float bj = 0.0f;
                    if (lane < cnt) {
                        cj4 = t.pos[cb + lane];
                        bj = ball2[cb + lane];
                        rel = box_lb(make_float3(cj4.x, cj4.y, cj4.z), qlo, qhi, L, per) <
                              fmaxf(bj, qlo.w);
                    }
                    const unsigned R = __ballot_sync(SKID_FULL, rel);
                    const int nR = __popc(R);
                    __syncwarp();
                    if (rel) {
                        const int k = __popc(R & ((1u << lane) - 1u));
                        float ih2 = 4.0f / bj;
                        cpos[w][k] = cj4;
                        caux[w][k] = make_float4(bj, ih2, 0.5f * (float)M_1_PI * sqrtf(ih2) * ih2, 0.0f);
                    }
                    __syncwarp();
                    if (!want) continue;
                    int cx = img_class(q.x, blo.x, bhi.x, hL.x);
                    int cy = img_class(q.y, blo.y, bhi.y, hL.y);
                    int cz = img_class(q.z, blo.z, bhi.z, hL.z);
                    bool mixed = (cx == 2) | (cy == 2) | (cz == 2);
                    bool noshift = (cx == 0) & (cy == 0) & (cz == 0);
                    float sx = shifted(q.x, cx, L.x), sy = shifted(q.y, cy, L.y), sz = shifted(q.z, cz, L.z);
                    for (int j = 0; j < nR; ++j) {
                        float4 cj = cpos[w][j];
                        float4 aj = caux[w][j];
                        float dik, dki;
                        if (mixed) {
                            dik = d2of(img_dx(q.x, cj.x, L.x, hL.x), img_dx(q.y, cj.y, L.y, hL.y),
                                       img_dx(q.z, cj.z, L.z, hL.z));
                            dki = d2of(img_dx(cj.x, q.x, L.x, hL.x), img_dx(cj.y, q.y, L.y, hL.y),
                                       img_dx(cj.z, q.z, L.z, hL.z));
                        } else {
                            dik = d2of(fsub(sx, cj.x), fsub(sy, cj.y), fsub(sz, cj.z));
                            if (noshift) {
                                dki = dik;
                            } else {
                                dki = d2of(fsub(shifted(cj.x, -cx, L.x), q.x),
                                           fsub(shifted(cj.y, -cy, L.y), q.y),
                                           fsub(shifted(cj.z, -cz, L.z), q.z));
                            }
                        }
                        if (dik < bi) kahan_add(s, c, cj.w * fni * w_m4(dik * ih2i));
                        if (dki < aj.x) kahan_add(s, c, cj.w * aj.z * w_m4(dki * aj.y));
                    }
                }
            } else {
                float4 blo = t.lo[cp], bhi = t.hi[cp];
                bool want = box_lb(q, blo, bhi, L, per) < fmaxf(bi, blo.w);
                if (__any_sync(SKID_FULL, want)) { cp <<= 1; continue; }
            }
            cp = next_node(cp);
            if (cp == 1) break;
        }
        if (valid) rho[qi] = s;
    }
}

// Movers per warp G: 64, 32, 16, 8, 4 or 1; with G <= 32, 32/G lanes per
// mover, and with G = 64 two movers per lane.  More movers per warp share
// the tree walk and the leaf staging among more of them while the active
// movers are dense; fewer keep the union of their neighbourhoods small when
// they are sparse.  At a visited leaf the candidates whose ball reaches the
// movers' box are compacted in order; a mover's lanes test every (32/G)-th
// of them (one cheap pass that sets a hit mask), then run the field terms for
// their hits only, and are combined with a fixed xor-butterfly, so sums are
// deterministic for a given G.
template <int G, bool STATS>
__global__ void __launch_bounds__(G_WARPS * 32, G > 32 ? 10 : SKID_FIELD_MINB)
field_kernel(FieldArgs a)
{
    constexpr int MPL = G > 32 ? G / 32 : 1;   // movers per lane
    constexpr int L = G >= 32 ? 1 : 32 / G;    // lanes per mover
    __shared__ float4 cpos_s[G_WARPS][SKID_LEAF];
    __shared__ float2 ccoef_s[G_WARPS][SKID_LEAF];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nA = *a.d_nA;
    const int nC = *a.d_nC;
    // One mover per warp and few movers: each mover's walk is split over S
    // warps (about FIELD_SPLIT_ITEMS warps in all); all walk the inner nodes,
    // and of each 32 leaves under a node, part p takes every S-th from p.
    int S = 1;
    if (G == 1 && a.part_acc && a.logLeafBase >= 5) {
        const int t = FIELD_SPLIT_ITEMS / (nA > 0 ? nA : 1);
        S = t >= 16 ? 16 : t >= 8 ? 8 : t >= 4 ? 4 : t >= 2 ? 2 : 1;
    }
    const int nItems = G == 1 ? nA * S : (nA + G - 1) / G;
    const int sub = lane % L;
    unsigned long long st_nodes = 0, st_leaves = 0, st_tests = 0, st_hits = 0;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.d_work, 1);
        item = __shfl_sync(SKID_FULL, item, 0);
        if (item >= nItems) break;
        int part = 0;
        if (G == 1) {
            part = item % S;
            item /= S;
        }
        int slot[MPL], mi[MPL];
        bool valid[MPL];
        float4 yp[MPL];
        float3 y[MPL];
        // bounding box of the warp's movers, for the per-leaf candidate prefilter
        float3 wlo = make_float3(FLT_MAX, FLT_MAX, FLT_MAX);
        float3 whi = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
#pragma unroll
        for (int k = 0; k < MPL; ++k) {
            slot[k] = item * G + k * 32 + lane / L;
            valid[k] = slot[k] < nA;
            mi[k] = a.act[valid[k] ? slot[k] : item * G];
            yp[k] = a.mpos[mi[k]];
            y[k] = make_float3(yp[k].x, yp[k].y, yp[k].z);
            if (valid[k]) {
                wlo = make_float3(fminf(wlo.x, y[k].x), fminf(wlo.y, y[k].y), fminf(wlo.z, y[k].z));
                whi = make_float3(fmaxf(whi.x, y[k].x), fmaxf(whi.y, y[k].y), fmaxf(whi.z, y[k].z));
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            wlo.x = fminf(wlo.x, __shfl_xor_sync(SKID_FULL, wlo.x, o));
            wlo.y = fminf(wlo.y, __shfl_xor_sync(SKID_FULL, wlo.y, o));
            wlo.z = fminf(wlo.z, __shfl_xor_sync(SKID_FULL, wlo.z, o));
            whi.x = fmaxf(whi.x, __shfl_xor_sync(SKID_FULL, whi.x, o));
            whi.y = fmaxf(whi.y, __shfl_xor_sync(SKID_FULL, whi.y, o));
            whi.z = fmaxf(whi.z, __shfl_xor_sync(SKID_FULL, whi.z, o));
        }
        float ax[MPL], ay[MPL], az[MPL];
#pragma unroll
        for (int k = 0; k < MPL; ++k) ax[k] = ay[k] = az[k] = 0.0f;
        // Depth-first walk by ball boxes in strides of five levels, aligned
        // so the last stride ends at the leaves: a visited node has each lane
        // test one of its 32 descendants five levels down against the movers'
        // box, and those that pass are visited in order (so leaves come in
        // depth-first order).  A visited node is entered only if some mover
        // lies in its ball box.  Stack level l (its first node and the
        // descendants still to visit) is held by lane l.
        auto reach = [&](int node) {
            float4 bl = a.blo[node], bh = a.bhi[node];
            return bl.x <= whi.x && bh.x >= wlo.x && bl.y <= whi.y && bh.y >= wlo.y &&
                   bl.z <= whi.z && bh.z >= wlo.z;
        };
        unsigned smask;
        int sfirst;
        {
            const int d0 = a.logLeafBase % 5;
            sfirst = 1 << d0;
            smask = __ballot_sync(SKID_FULL, lane < (1 << d0) && reach(sfirst + lane));
        }
        int sp = 0;
        while (sp >= 0) {
            const unsigned m = __shfl_sync(SKID_FULL, smask, sp);
            if (!m) { --sp; continue; }
            const int node = __shfl_sync(SKID_FULL, sfirst, sp) + __ffs(m) - 1;
            if (lane == sp) smask = m & (m - 1);
            if (STATS) ++st_nodes;
            {
                float4 blo = a.blo[node], bhi = a.bhi[node];
                bool want = false;
#pragma unroll
                for (int k = 0; k < MPL; ++k)
                    want = want || (valid[k] && y[k].x >= blo.x && y[k].x <= bhi.x &&
                                    y[k].y >= blo.y && y[k].y <= bhi.y && y[k].z >= blo.z &&
                                    y[k].z <= bhi.z);
                if (!__any_sync(SKID_FULL, want)) continue;
                if (node < a.leafBase) {
                    const int cf = node << 5;
                    unsigned cm = __ballot_sync(SKID_FULL, reach(cf + lane));
                    if (G == 1 && S > 1 && cf >= a.leafBase)
                        cm &= (S == 2 ? 0x55555555u : S == 4 ? 0x11111111u
                               : S == 8 ? 0x01010101u : 0x00010001u) << part;
                    if (cm) {
                        ++sp;
                        if (lane == sp) { smask = cm; sfirst = cf; }
                    }
                    continue;
                }
                int cb = (node - a.leafBase) * SKID_LEAF;
                int cnt = min(SKID_LEAF, nC - cb);
                if (STATS) ++st_leaves;
                // prefilter: lane j keeps candidate j if its ball (radius
                // rounded up) reaches the movers' box; the exact test below
                // decides, so this only skips candidates that cannot hit
                bool rel = false;
                float4 c4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (lane < cnt) {
                    c4 = a.cpos[cb + lane];
                    // ball radius from the approximate reciprocal square root,
                    // widened to cover its error (an empty ball, fBall2 = 0,
                    // gives NaN and is rejected, as the exact test would)
                    float r = c4.w * rsqrtf(c4.w) * (1.0f + 4e-6f) +
                              1e-6f * (fabsf(c4.x) + fabsf(c4.y) + fabsf(c4.z)) + 1e-30f;
                    // the ball itself against the box: squared distance from
                    // the copy to the movers' box (per-axis gaps, zero inside)
                    const float gx = fmaxf(fmaxf(wlo.x - c4.x, c4.x - whi.x), 0.0f);
                    const float gy = fmaxf(fmaxf(wlo.y - c4.y, c4.y - whi.y), 0.0f);
                    const float gz = fmaxf(fmaxf(wlo.z - c4.z, c4.z - whi.z), 0.0f);
                    rel = __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, gx * gx)) <= r * r;
                }
                // the survivors, compacted in candidate order
                const unsigned R = __ballot_sync(SKID_FULL, rel);
                const int nR = __popc(R);
                const int slotR = __popc(R & ((1u << lane) - 1u));
                __syncwarp();
                if (rel) {
                    cpos_s[w][slotR] = c4;
                    float4 cc = a.ccoef[cb + lane];
                    ccoef_s[w][slotR] = make_float2(cc.x, cc.y);
                }
                __syncwarp();
                // a mover's L lanes take every L-th survivor
                unsigned mask[MPL];
#pragma unroll
                for (int k = 0; k < MPL; ++k) mask[k] = 0;
                if (want) {
#pragma unroll FIELD_UNROLL
                    for (int t = sub; t < nR; t += L) {
                        float4 c = cpos_s[w][t];
#pragma unroll
                        for (int k = 0; k < MPL; ++k) {
                            // smBallGather's test (smooth1.c:365-369), from the copy
                            float d2 = d2of(fsub(c.x, y[k].x), fsub(c.y, y[k].y), fsub(c.z, y[k].z));
                            mask[k] |= (unsigned)(d2 < c.w) << t;
                        }
                    }
                    if (STATS) st_tests += MPL * ((nR - sub + L - 1) / L);
                }
                unsigned hitany = 0;
#pragma unroll
                for (int k = 0; k < MPL; ++k) {
                    hitany |= mask[k];
                    if (STATS) st_hits += __popc(mask[k]);
                    for (unsigned m = mask[k]; m; m &= m - 1) {
                        int j = __ffs(m) - 1;
                        float4 c = cpos_s[w][j];
                        float2 cf = ccoef_s[w][j];
                        // the field value (smooth1.c:450-458) only has to be
                        // accurate, not bit-exact: FMA and the approximate
                        // reciprocal square root (q = r2 / sqrt(r2), 1/q)
                        float dx = c.x - y[k].x, dy = c.y - y[k].y, dz = c.z - y[k].z;
                        float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx)) * cf.x;
                        float iq = rsqrtf(r2);
                        float q = r2 > 0.0f ? r2 * iq : 0.0f;
                        float F = r2 < 1.0f ? __fmaf_rn(2.25f, q, -3.0f)
                                            : __fmaf_rn(-0.75f, q, 3.0f) - 3.0f * iq;
                        F *= cf.y;
                        ax[k] = __fmaf_rn(dx, F, ax[k]);
                        ay[k] = __fmaf_rn(dy, F, ay[k]);
                        az[k] = __fmaf_rn(dz, F, az[k]);
                    }
                }
                // copies that reached a mover: touched, and their density
                // enters the floor of the cut (smooth1.c:460-461)
                unsigned any = __reduce_or_sync(SKID_FULL, hitany);
                if (rel && ((any >> slotR) & 1u)) a.touched[cb + lane] = 1;
            }
        }
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) {
            ax[0] = fadd(ax[0], __shfl_xor_sync(SKID_FULL, ax[0], o));
            ay[0] = fadd(ay[0], __shfl_xor_sync(SKID_FULL, ay[0], o));
            az[0] = fadd(az[0], __shfl_xor_sync(SKID_FULL, az[0], o));
        }
        if (sub != 0) continue;
#pragma unroll
        for (int k = 0; k < MPL; ++k) {
            if (!valid[k]) continue;
            float fx = ax[k], fy = ay[k], fz = az[k];
            if (G == 1 && S > 1) {
                // the last of the mover's S parts sums them in part order
                float *pa = a.part_acc + 3 * ((size_t)slot[k] * S + part);
                pa[0] = fx;
                pa[1] = fy;
                pa[2] = fz;
                __threadfence();
                if (atomicAdd(&a.part_cnt[slot[k]], 1) != S - 1) continue;
                __threadfence();
                fx = fy = fz = 0.0f;
                for (int p = 0; p < S; ++p) {
                    const float *q = a.part_acc + 3 * ((size_t)slot[k] * S + p);
                    fx = fadd(fx, __ldcg(q));
                    fy = fadd(fy, __ldcg(q + 1));
                    fz = fadd(fz, __ldcg(q + 2));
                }
                a.part_cnt[slot[k]] = 0;
            }
            if (a.acc_out) {
                a.acc_out[3 * (size_t)slot[k] + 0] = fx;
                a.acc_out[3 * (size_t)slot[k] + 1] = fy;
                a.acc_out[3 * (size_t)slot[k] + 2] = fz;
            }
            if (a.fStep > 0.0f) {
                // kdMoveParticles (kd.c:711-728)
                float3 yk = y[k];
                float s2 = d2of(fx, fy, fz);
                float ai = sqrtf(s2);
                ai = ai > 0.0f ? __fdiv_rn(a.fStep, ai) : 0.0f;
                yk.x = fsub(yk.x, fmul(ai, fx));
                yk.y = fsub(yk.y, fmul(ai, fy));
                yk.z = fsub(yk.z, fmul(ai, fz));
                if (yk.x > a.wrapHi.x) yk.x = fsub(yk.x, a.period.x);
                if (yk.x <= a.wrapLo.x) yk.x = fadd(yk.x, a.period.x);
                if (yk.y > a.wrapHi.y) yk.y = fsub(yk.y, a.period.y);
                if (yk.y <= a.wrapLo.y) yk.y = fadd(yk.y, a.period.y);
                if (yk.z > a.wrapHi.z) yk.z = fsub(yk.z, a.period.z);
                if (yk.z <= a.wrapLo.z) yk.z = fadd(yk.z, a.period.z);
                a.mpos[mi[k]] = make_float4(yk.x, yk.y, yk.z, yp[k].w);
            }
        }
    }
    if (STATS && a.stats) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            st_tests += __shfl_xor_sync(SKID_FULL, st_tests, o);
            st_hits += __shfl_xor_sync(SKID_FULL, st_hits, o);
        }
        if (lane == 0) {
            atomicAdd(&a.stats[0], st_nodes);
            atomicAdd(&a.stats[1], st_leaves);
            atomicAdd(&a.stats[2], st_tests);
            atomicAdd(&a.stats[3], st_hits);
        }
    }
}

}  // namespace

cudaError_t density_gather(const Tree &t, const float *ball2_sorted, float3 L, bool per,
                           float *rho_sorted, int *d_work, cudaStream_t st)
{
    if (t.n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_work, 0, sizeof(int), st);
    if (e) return e;
    int perSM = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, density_kernel, G_WARPS * 32, 0);
    if (perSM < 1) perSM = 1;
    int blocks = num_sms() * perSM;
    int need = (t.nLeaf + G_WARPS - 1) / G_WARPS;
    if (blocks > need) blocks = need;
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    int subShift = 0;
    while (subShift < 5 && (2 << subShift) <= t.leafBase) ++subShift;
    density_kernel<<<blocks, G_WARPS * 32, 0, st>>>(t.view(), ball2_sorted, L, hL, per, subShift,
                                                    rho_sorted, d_work); skid::note_launch();
    return cudaGetLastError();
}

template <int G, bool STATS>
static cudaError_t launch_field_t(const FieldArgs &a, int max_movers, cudaStream_t st)
{
    int perSM = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, field_kernel<G, STATS>, G_WARPS * 32, 0);
    if (perSM < 1) perSM = 1;
    int blocks = num_sms() * perSM;
    int need = ((max_movers + G - 1) / G + G_WARPS - 1) / G_WARPS;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    field_kernel<G, STATS><<<blocks, G_WARPS * 32, 0, st>>>(a); skid::note_launch();
    return cudaGetLastError();
}

// Work counters compiled in only when asked for (they cost registers).
template <int G>
static cudaError_t launch_field(const FieldArgs &a, int max_movers, cudaStream_t st)
{
    return a.stats ? launch_field_t<G, true>(a, max_movers, st) : launch_field_t<G, false>(a, max_movers, st);
}

// The move alone (kdMoveParticles, kd.c:702-732) from a field written by
// field_kernel with fStep = 0: the unfused form, a separate gradient pass.
__global__ void move_kernel(FieldArgs a, const float *__restrict__ acc, float fStep, int cap)
{
    const int nA = *a.d_nA;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nA && slot < cap;
         slot += gridDim.x * blockDim.x) {
        int mi = a.act[slot];
        if (mi < 0 || mi >= cap) {
            set_status(a.d_status, ST_BADSTATE);
            continue;
        }
        float4 yp = a.mpos[mi];
        float3 y = make_float3(yp.x, yp.y, yp.z);
        float ax = acc[3 * (size_t)slot], ay = acc[3 * (size_t)slot + 1], az = acc[3 * (size_t)slot + 2];
        float s = d2of(ax, ay, az);
        float ai = sqrtf(s);
        ai = ai > 0.0f ? __fdiv_rn(fStep, ai) : 0.0f;
        y.x = fsub(y.x, fmul(ai, ax));
        y.y = fsub(y.y, fmul(ai, ay));
        y.z = fsub(y.z, fmul(ai, az));
        if (y.x > a.wrapHi.x) y.x = fsub(y.x, a.period.x);
        if (y.x <= a.wrapLo.x) y.x = fadd(y.x, a.period.x);
        if (y.y > a.wrapHi.y) y.y = fsub(y.y, a.period.y);
        if (y.y <= a.wrapLo.y) y.y = fadd(y.y, a.period.y);
        if (y.z > a.wrapHi.z) y.z = fsub(y.z, a.period.z);
        if (y.z <= a.wrapLo.z) y.z = fadd(y.z, a.period.z);
        a.mpos[mi] = make_float4(y.x, y.y, y.z, yp.w);
    }
}

cudaError_t move_movers(const FieldArgs &a, const float *acc, float fStep, int max_movers,
                        cudaStream_t st)
{
    if (max_movers <= 0) return cudaSuccess;
    move_kernel<<<grid_for(max_movers), 256, 0, st>>>(a, acc, fStep, max_movers); note_launch();
    return cudaGetLastError();
}

cudaError_t field_move(const FieldArgs &a, int max_movers, cudaStream_t st)
{
    if (max_movers <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.d_work, 0, sizeof(int), st);
    if (e) return e;
    switch (a.G) {
    case 64: return launch_field<64>(a, max_movers, st);
    case 1: return launch_field<1>(a, max_movers, st);
    case 4: return launch_field<4>(a, max_movers, st);
    case 8: return launch_field<8>(a, max_movers, st);
    case 16: return launch_field<16>(a, max_movers, st);
    default: return launch_field<32>(a, max_movers, st);
    }
}

}  // namespace skid
