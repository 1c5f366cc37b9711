// Group bookkeeping on the device.
//
//  - group_order: particles sorted by group id (stable, so members of a group
//    are in ascending iOrder), with start/count per group -- the role of
//    kdGroupOrder (kd.c:1205-1245).
//  - group_props: kdInitpGroup (kd.c:969-1005) + kdCalcCenter
//    (kd.c:1013-1075): members, mass, reference point rel (the smallest-iOrder
//    member after a move; any member gives the same centre up to rounding),
//    density centre = rel + mean of the wrapped moved offsets, mass-weighted
//    mean velocity.  With `com` set it is kdReadCenter's fallback
//    (kd.c:1160-1192): mass-weighted centre of the input positions.  With
//    `rel_last` rel is the largest-iOrder member, as kdInitpGroup leaves it
//    when the groups are read from a file (its loop runs in iOrder there).
//  - too_small: kdTooSmall (kd.c:1251-1293), order-preserving renumbering.
//  - group_radius: max distance of current members from the centre
//    (kdWriteGroup, kd.c:1627-1644).
#include <cfloat>

#include "ctx.h"

namespace skid {

namespace {

__global__ void keys_from_groups(const int *__restrict__ grp, int n, uint64_t *keys, uint32_t *vals)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = (uint64_t)(uint32_t)grp[i];
        vals[i] = (uint32_t)i;
    }
}

// start[g] = first slot; count[g] temporarily holds the end slot.
__global__ void group_bounds(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                             int n, int ng, int *__restrict__ start, int *__restrict__ count,
                             int *__restrict__ members, int *__restrict__ gof)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int g = (int)keys[i];
        members[i] = (int)vals[i];
        gof[i] = g;
        if (i == 0 || (int)keys[i - 1] != g) start[g] = i;
        if (i == n - 1 || (int)keys[i + 1] != g) count[g] = i + 1;
    }
}

__global__ void group_counts(int *__restrict__ start, int *__restrict__ count, int ng)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int s = start[g];
        if (s < 0) { start[g] = 0; count[g] = 0; continue; }
        count[g] = count[g] - s;
    }
}

__device__ __forceinline__ float wrap_half(float d, float h, float L)
{
    // kd.c:1037-1039: if (del > 0.5*fPeriod) del -= fPeriod; if (del <= -0.5*fPeriod) del += fPeriod
    if (d > h) d = fsub(d, L);
    if (d <= -h) d = fadd(d, L);
    return d;
}

// One warp per group.
__global__ void group_props_kernel(const int *__restrict__ start, const int *__restrict__ count,
                                   const int *__restrict__ members, int ng,
                                   const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                                   const float4 *__restrict__ moved, float3 L, float3 hL,
                                   float3 wrapHi, float3 wrapLo, int com, int rel_last,
                                   skid_group *__restrict__ rec)
{
    int lane = threadIdx.x & 31;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nw = (gridDim.x * blockDim.x) >> 5;
    for (int g = warp; g < ng; g += nw) {
        int s = start[g], c = count[g];
        skid_group r = rec[g];
        r.nMembers = c;
        if (g == 0 || c == 0) {
            if (lane == 0) {
                if (g == 0) {
                    r.fMass = 0.0f;
                    for (int d = 0; d < 3; ++d) r.rel[d] = r.rCenter[d] = r.rBound[d] = r.vcm[d] = 0.0f;
                    r.fRadius = 0.0f;
                }
                rec[g] = r;
            }
            continue;
        }
        float4 rp = pos4[members[rel_last ? s + c - 1 : s]];
        float rel[3] = {rp.x, rp.y, rp.z};
        double m = 0.0, cs[3] = {0, 0, 0}, vs[3] = {0, 0, 0};
        for (int k = s + lane; k < s + c; k += 32) {
            int io = members[k];
            float4 p = pos4[io];
            float4 v = vel4[io];
            float4 q = com ? p : moved[io];
            m += p.w;
            float del0 = wrap_half(fsub(q.x, rel[0]), hL.x, L.x);
            float del1 = wrap_half(fsub(q.y, rel[1]), hL.y, L.y);
            float del2 = wrap_half(fsub(q.z, rel[2]), hL.z, L.z);
            if (com) {
                cs[0] += fmul(p.w, del0); cs[1] += fmul(p.w, del1); cs[2] += fmul(p.w, del2);
            } else {
                cs[0] += del0; cs[1] += del1; cs[2] += del2;
            }
            vs[0] += fmul(p.w, v.x); vs[1] += fmul(p.w, v.y); vs[2] += fmul(p.w, v.z);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            m += __shfl_xor_sync(SKID_FULL, m, o);
            for (int d = 0; d < 3; ++d) {
                cs[d] += __shfl_xor_sync(SKID_FULL, cs[d], o);
                vs[d] += __shfl_xor_sync(SKID_FULL, vs[d], o);
            }
        }
        if (lane == 0) {
            float fm = (float)m;
            r.fMass = fm;
            float wh[3] = {wrapHi.x, wrapHi.y, wrapHi.z}, wl[3] = {wrapLo.x, wrapLo.y, wrapLo.z};
            float Ld[3] = {L.x, L.y, L.z};
            for (int d = 0; d < 3; ++d) {
                r.rel[d] = rel[d];
                float cc = (float)cs[d];
                cc = com ? cc / fm : cc / (float)c;
                cc = fadd(cc, rel[d]);
                if (cc > wh[d]) cc = fsub(cc, Ld[d]);
                if (cc <= wl[d]) cc = fadd(cc, Ld[d]);
                r.rCenter[d] = cc;
                r.vcm[d] = (float)vs[d] / fm;
                r.rBound[d] = 0.0f;
            }
            r.fRadius = 0.0f;
            rec[g] = r;
        }
    }
}

__global__ void toosmall_flags(const skid_group *__restrict__ rec, int ng, int nmin,
                               int *__restrict__ flag)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int c = rec[g].nMembers;
        flag[g] = g > 0 && c >= nmin && c > 0;
    }
}

__global__ void toosmall_apply(const int *__restrict__ flag, const int *__restrict__ rank, int ng,
                               const skid_group *__restrict__ rec, skid_group *__restrict__ rec2,
                               int *__restrict__ map)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        if (g == 0) { map[0] = 0; rec2[0] = rec[0]; continue; }
        if (flag[g]) {
            int k = rank[g] + 1;
            map[g] = k;
            rec2[k] = rec[g];
        } else {
            map[g] = 0;
        }
    }
}

__global__ void remap_groups(int *__restrict__ grp, int n, const int *__restrict__ map)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        grp[i] = map[grp[i]];
}

__global__ void radius_kernel(const int *__restrict__ grp, int n, const float4 *__restrict__ pos4,
                              const skid_group *__restrict__ rec, float3 L, float3 hL,
                              unsigned *__restrict__ rmax)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int g = grp[i];
        if (!g) continue;
        float4 p = pos4[i];
        const float *c = rec[g].rCenter;
        float d0 = wrap_half(fsub(p.x, c[0]), hL.x, L.x);
        float d1 = wrap_half(fsub(p.y, c[1]), hL.y, L.y);
        float d2 = wrap_half(fsub(p.z, c[2]), hL.z, L.z);
        float r = sqrtf(d2of(d0, d1, d2));
        atomicMax(&rmax[g], __float_as_uint(r));
    }
}

__global__ void radius_store(const unsigned *__restrict__ rmax, int ng, skid_group *__restrict__ rec)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
        rec[g].fRadius = g ? __uint_as_float(rmax[g]) : 0.0f;
}

__global__ void fill_int(int *p, int v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

int bits_for(int v)
{
    int b = 1;
    while ((1ll << b) <= v) ++b;
    return (b + 7) & ~7;
}

}  // namespace

cudaError_t group_order(const int *grp, int n, int ng, SortScratch &ss, GroupState &G,
                        cudaStream_t st)
{
    cudaError_t e;
    if ((e = dalloc(ss.k0, n)) || (e = dalloc(ss.k1, n)) || (e = dalloc(ss.v0, n)) ||
        (e = dalloc(ss.v1, n)) || (e = dalloc(G.members, n)) || (e = dalloc(G.start, ng)) ||
        (e = dalloc(G.count, ng)) || (e = dalloc(G.gof, n)))
        return e;
    keys_from_groups<<<grid_for(n), 256, 0, st>>>(grp, n, ss.k0.p, ss.v0.p); skid::note_launch();
    if ((e = radix_sort(ss, n, bits_for(ng), st))) return e;
    fill_int<<<grid_for(ng), 256, 0, st>>>(G.start.p, -1, ng); skid::note_launch();
    group_bounds<<<grid_for(n), 256, 0, st>>>(ss.k0.p, ss.v0.p, n, ng, G.start.p, G.count.p,
                                              G.members.p, G.gof.p); skid::note_launch();
    group_counts<<<grid_for(ng), 256, 0, st>>>(G.start.p, G.count.p, ng); skid::note_launch();
    return cudaGetLastError();
}

cudaError_t group_props(GroupState &G, const float4 *pos4, const float4 *vel4, const float4 *moved,
                        float3 L, float3 wrapHi, float3 wrapLo, bool com, bool rel_last,
                        cudaStream_t st)
{
    cudaError_t e;
    if ((e = dalloc(G.rec, G.nGroup))) return e;
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    int warps = G.nGroup;
    int blocks = min((warps * 32 + 255) / 256, num_sms() * 16);
    if (blocks < 1) blocks = 1;
    group_props_kernel<<<blocks, 256, 0, st>>>(G.start.p, G.count.p, G.members.p, G.nGroup, pos4,
                                               vel4, moved, L, hL, wrapHi, wrapLo, com ? 1 : 0,
                                               rel_last ? 1 : 0, G.rec.p); skid::note_launch();
    return cudaGetLastError();
}

cudaError_t too_small(GroupState &G, int *grp, int n, int nmin, int *d_ng, SortScratch &ss,
                      cudaStream_t st)
{
    cudaError_t e;
    int ng = G.nGroup;
    if ((e = dalloc(G.gtmp, ng)) || (e = dalloc(G.gtmp2, ng)) || (e = dalloc(G.map, ng)))
        return e;
    if ((e = dalloc(G.rec2, ng))) return e;
    toosmall_flags<<<grid_for(ng), 256, 0, st>>>(G.rec.p, ng, nmin, G.gtmp.p); skid::note_launch();
    if ((e = scan_exclusive(G.gtmp.p, G.gtmp2.p, ng, d_ng, ss, st))) return e;
    // rank[g] = position among kept groups; records move to slot rank+1
    toosmall_apply<<<grid_for(ng), 256, 0, st>>>(G.gtmp.p, G.gtmp2.p, ng, G.rec.p, G.rec2.p,
                                                 G.map.p); skid::note_launch();
    if ((e = cudaMemcpyAsync(G.rec.p, G.rec2.p, ng * sizeof(skid_group), cudaMemcpyDeviceToDevice,
                             st)))
        return e;
    remap_groups<<<grid_for(n), 256, 0, st>>>(grp, n, G.map.p); skid::note_launch();
    return cudaGetLastError();
}

cudaError_t group_radius(GroupState &G, const int *grp, int n, const float4 *pos4, float3 L,
                         cudaStream_t st)
{
    cudaError_t e;
    int ng = G.nGroup;
    if ((e = dalloc(G.gtmp, ng))) return e;
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    if ((e = cudaMemsetAsync(G.gtmp.p, 0, ng * sizeof(int), st))) return e;
    radius_kernel<<<grid_for(n), 256, 0, st>>>(grp, n, pos4, G.rec.p, L, hL, (unsigned *)G.gtmp.p); skid::note_launch();
    radius_store<<<grid_for(ng), 256, 0, st>>>((const unsigned *)G.gtmp.p, ng, G.rec.p); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
