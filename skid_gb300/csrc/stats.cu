// Per-group statistics of the .stat table (kdOutStats, kd.c:1703-1839) on the
// device, after too-small removal.
//
// The reference takes each group's members relative to its density centre
// (wrapped with half periods), sorts them by radius with qsort, and walks
// them outwards keeping running float sums: total, gas and star mass, the
// largest G M(<r)/r outside twice the softening, the radius where the
// enclosed mass first exceeds half, and the velocity dispersion about vcm
// with the Hubble flow.  Here:
//   1. one thread per particle forms the key (group << 32 | radius^2 bits;
//      radius^2 >= 0, so its bits order like its value) -- ungrouped
//      particles get the largest key;
//   2. a stable radix sort of (key, iOrder) puts every group's members in
//      radius order, ties in iOrder order;
//   3. one thread per sorted slot marks where each group's run starts;
//   4. one thread per group walks its run outwards with the reference's own
//      float and double operations, each rounded as gcc rounds it, so the
//      running sums and the maximum / half-mass decisions are the
//      reference's (the sums are inherently sequential: each depends on the
//      float rounding of the previous one).
#include <cfloat>

#include "ctx.h"

using namespace skid;

namespace {

__device__ __forceinline__ float stat_wrap(float d, float h)
{
    // kd.c:1741-1746: if (dx > hx) dx -= 2*hx; if (dx <= -hx) dx += 2*hx
    if (d > h) d = fsub(d, fmul(2.0f, h));
    if (d <= -h) d = fadd(d, fmul(2.0f, h));
    return d;
}

__device__ __forceinline__ float3 stat_rel(float4 p, const skid_group &g, float3 h)
{
    return make_float3(stat_wrap(fsub(p.x, g.rCenter[0]), h.x),
                       stat_wrap(fsub(p.y, g.rCenter[1]), h.y),
                       stat_wrap(fsub(p.z, g.rCenter[2]), h.z));
}

__global__ void stat_keys(const float4 *__restrict__ pos4, const int *__restrict__ grp, int n,
                          const skid_group *__restrict__ rec, float3 h, uint64_t *__restrict__ keys,
                          uint32_t *__restrict__ vals)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int g = grp[i];
        uint64_t k = ~0ull;
        if (g > 0) {
            const float3 r = stat_rel(pos4[i], rec[g], h);
            // kd.c:1756-1760: radius2 = 0.0; radius2 += r_k * r_k (float)
            const float r2 = fadd(fadd(fmul(r.x, r.x), fmul(r.y, r.y)), fmul(r.z, r.z));
            k = ((uint64_t)(unsigned)g << 32) | __float_as_uint(r2);
        }
        keys[i] = k;
        vals[i] = (uint32_t)i;
    }
}

__global__ void stat_starts(const uint64_t *__restrict__ keys, int n, int *__restrict__ start)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint64_t k = keys[p];
        if (k == ~0ull) continue;
        const unsigned g = (unsigned)(k >> 32);
        if (p == 0 || (unsigned)(keys[p - 1] >> 32) != g) start[g] = p;
    }
}

struct StatArgs {
    const uint64_t *keys;
    const uint32_t *vals;
    const int *start;
    const skid_group *rec;
    const float4 *pos4, *vel4;
    const float *temp, *rho;
    int nGroup, nGas, nDark;
    float3 h;
    float G, fExp, fExpHub, fDensMin, fTempMax;
    skid_stat *out;
};

__global__ void stat_groups(StatArgs A)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x + 1; g < A.nGroup;
         g += gridDim.x * blockDim.x) {
        const skid_group rg = A.rec[g];
        const int n = rg.nMembers, s = A.start[g];
        skid_stat o;
        o.nMembers = n;
        if (n <= 0) {
            o.fTotMass = o.fGasMass = o.fStarMass = 0.0f;
            o.fVcirc2Max = o.fVcirc2Half = o.fVcirc2Outer = 0.0f;
            o.fRVmax = o.fRHalf = o.fROuter2 = o.fVdisp = 0.0f;
            A.out[g] = o;
            continue;
        }
        // kd.c:1766-1767: fHalfMass += 0.5*fMass (FP64 sum rounded to float)
        float fHalf = 0.0f;
        for (int j = 0; j < n; ++j)
            fHalf = (float)__dadd_rn((double)fHalf, __dmul_rn(0.5, (double)A.pos4[A.vals[s + j]].w));
        float fTot = 0.0f, fGas = 0.0f, fStar = 0.0f, fVc = 0.0f, fmVc = 0.0f, fVd = 0.0f;
        float fRVmax = 0.0f, fRh = 0.0f, r2 = 0.0f;
        for (int j = 0; j < n; ++j) {
            const int io = (int)A.vals[s + j];
            const float4 p = A.pos4[io], v = A.vel4[io];
            r2 = __uint_as_float((unsigned)A.keys[s + j]);
            const float m = p.w, soft = v.w;
            fTot = fadd(fTot, m);
            // kd.c:1774-1778: r2 > 4.0*soft*soft && G*fTot/sqrt(r2) > fVcirc
            // (FP64 comparisons); fRVmax = sqrt(r2), fVcirc = G*fTot/fRVmax (float)
            const double d2 = (double)r2;
            if (d2 > __dmul_rn(__dmul_rn(4.0, (double)soft), (double)soft) &&
                __ddiv_rn((double)fmul(A.G, fTot), __dsqrt_rn(d2)) > (double)fVc) {
                fRVmax = (float)__dsqrt_rn(d2);
                fVc = __fdiv_rn(fmul(A.G, fTot), fRVmax);
            }
            const bool gas = io < A.nGas, star = io >= A.nGas + A.nDark;
            if (gas && A.rho[io] >= A.fDensMin && A.temp[io] <= A.fTempMax) fGas = fadd(fGas, m);
            if (star) fStar = fadd(fStar, m);
            if (fTot > fHalf && fmVc == 0.0f) {
                fRh = (float)__dsqrt_rn(d2);
                fmVc = __fdiv_rn(fmul(A.G, fTot), fRh);
            }
            const float3 r = stat_rel(p, rg, A.h);
            const float vv[3] = {v.x, v.y, v.z}, rr[3] = {r.x, r.y, r.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                // kd.c:1792-1796: dv = fExp*(v - vcm) + fExpHub*r (float)
                const float dv = fadd(fmul(A.fExp, fsub(vv[k], rg.vcm[k])), fmul(A.fExpHub, rr[k]));
                fVd = fadd(fVd, fmul(dv, dv));
            }
        }
        // kd.c:1798-1803: r2 is the outermost member's
        const float flVc = (float)__ddiv_rn((double)fmul(A.G, fTot), __dsqrt_rn((double)r2));
        if (fVc == 0.0f) {
            fVc = flVc;
            fRVmax = (float)__dsqrt_rn((double)r2);
        }
        fVd = (float)__dsqrt_rn(__ddiv_rn((double)fVd, __dmul_rn(3.0, (double)n)));
        o.fTotMass = fTot;
        o.fGasMass = fGas;
        o.fStarMass = fStar;
        o.fVcirc2Max = fVc;
        o.fVcirc2Half = fmVc;
        o.fVcirc2Outer = flVc;
        o.fRVmax = fRVmax;
        o.fRHalf = fRh;
        o.fROuter2 = r2;
        o.fVdisp = fVd;
        A.out[g] = o;
    }
}

int bits_for_groups(int ng)
{
    int b = 1;
    while (b < 31 && (1 << b) <= ng) ++b;
    return b;
}

}  // namespace

extern "C" int skid_group_stats(skid_ctx *ctx, float G, float fExp, float fExpHub, float fDensMin,
                                float fTempMax, skid_stat *stats)
{
    if (!ctx || !stats) return SKID_EINVAL;
    if (ctx->stage < STAGE_FINAL) return ctx->fail(SKID_ESTATE);
    const int n = ctx->n, ng = ctx->G.nGroup;
    cudaStream_t st = ctx->st;
    SortScratch &ss = ctx->ss;
    if (dalloc(ss.k0, n) || dalloc(ss.k1, n) || dalloc(ss.v0, n) || dalloc(ss.v1, n) ||
        dalloc(ctx->stat_start, ng > 0 ? ng : 1) || dalloc(ctx->stat_out, ng > 0 ? ng : 1))
        return ctx->fail(SKID_ENOMEM);
    if (ng <= 1) return 0;
    const float3 h = make_float3((float)(0.5 * (double)ctx->L.x), (float)(0.5 * (double)ctx->L.y),
                                 (float)(0.5 * (double)ctx->L.z));
    if (n > 0) {
        stat_keys<<<grid_for(n), 256, 0, st>>>(ctx->pos4.p, ctx->grp.p, n, ctx->G.rec.p, h,
                                               ss.k0.p, ss.v0.p); note_launch();
        CK(radix_sort(ss, n, 32 + bits_for_groups(ng), st));
        CK(cudaMemsetAsync(ctx->stat_start.p, 0, ng * sizeof(int), st));
        stat_starts<<<grid_for(n), 256, 0, st>>>(ss.k0.p, n, ctx->stat_start.p); note_launch();
    }
    StatArgs A;
    A.keys = ss.k0.p;
    A.vals = ss.v0.p;
    A.start = ctx->stat_start.p;
    A.rec = ctx->G.rec.p;
    A.pos4 = ctx->pos4.p;
    A.vel4 = ctx->vel4.p;
    A.temp = ctx->temp.p;
    A.rho = ctx->rho_final.p;
    A.nGroup = ng;
    A.nGas = ctx->nGas;
    A.nDark = ctx->nDark;
    A.h = h;
    A.G = G;
    A.fExp = fExp;
    A.fExpHub = fExpHub;
    A.fDensMin = fDensMin;
    A.fTempMax = fTempMax;
    A.out = ctx->stat_out.p;
    stat_groups<<<(ng + 127) / 128, 128, 0, st>>>(A); note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(stats, ctx->stat_out.p, ng * sizeof(skid_stat), cudaMemcpyDeviceToHost, st));
    return ctx->sync_check();
}
