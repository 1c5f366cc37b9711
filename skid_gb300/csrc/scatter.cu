// Scatterer and mover bookkeeping between move steps.
//
//  - scatter_aux: per scatterer the move-field coefficients and the set of
//    its copies: the original (bit 13) plus every periodic image whose
//    distance to the box is below fBall2 (the replicas of smooth1.c:283-332,
//    INTERSECTNP kd.h:102-119, same float arithmetic).
//  - cut: the heuristic scatterer removal (smooth1.c:460-470, 387-405,
//    509-513).  fScatDens = min density over copies that reached an active
//    mover; copies below it go.  On the first step (dark-only input or -fic)
//    copies that reached no mover count as density 0.  Surviving scatterers
//    are compacted in place order, which keeps them Morton-sorted.
//  - prune: kdPruneInactive (kd.c:735-793), stable.
#include <cfloat>

#include "internal.h"

namespace skid {

namespace {

constexpr unsigned ORIG_BIT = 13;

__global__ void aux_kernel(const float4 *__restrict__ spos, const float *__restrict__ ball2,
                           int n, float3 L, float3 blo, float3 bhi, int periodic,
                           float4 *__restrict__ aux, int *d_extra)
{
    int extra = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = spos[i];
        float b = ball2[i];
        unsigned m = 1u << ORIG_BIT;
        if (periodic) {
            for (int ix = -1; ix <= 1; ++ix)
                for (int iy = -1; iy <= 1; ++iy)
                    for (int iz = -1; iz <= 1; ++iz) {
                        if (!(ix | iy | iz)) continue;
                        float x = fadd(p.x, fmul((float)ix, L.x));
                        float y = fadd(p.y, fmul((float)iy, L.y));
                        float z = fadd(p.z, fmul((float)iz, L.z));
                        float dx = fsub(blo.x, x), dx1 = fsub(x, bhi.x);
                        float dy = fsub(blo.y, y), dy1 = fsub(y, bhi.y);
                        float dz = fsub(blo.z, z), dz1 = fsub(z, bhi.z);
                        float f;
                        if (dx > 0.0f) f = fmul(dx, dx);
                        else if (dx1 > 0.0f) f = fmul(dx1, dx1);
                        else f = 0.0f;
                        if (dy > 0.0f) f = fadd(f, fmul(dy, dy));
                        else if (dy1 > 0.0f) f = fadd(f, fmul(dy1, dy1));
                        if (dz > 0.0f) f = fadd(f, fmul(dz, dz));
                        else if (dz1 > 0.0f) f = fadd(f, fmul(dz1, dz1));
                        if (f < b) m |= 1u << ((ix + 1) * 9 + (iy + 1) * 3 + (iz + 1));
                    }
        }
        // smooth1.c:447-448: ih2 = 4/fBall2 (float); fNorm = M_1_PI ih2^2 sqrt(ih2) m
        float ih2 = (float)(4.0 / (double)b);
        double dih2 = ih2;
        float fnm = (float)(M_1_PI * dih2 * dih2 * sqrt(dih2) * (double)p.w);
        aux[i] = make_float4(b, ih2, fnm, __uint_as_float(m));
        extra += __popc(m) - 1;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) extra += __shfl_xor_sync(SKID_FULL, extra, o);
    if ((threadIdx.x & 31) == 0 && extra) atomicAdd(d_extra, extra);
}

// Pass 1 of the cut: density floor over touched live copies.
__global__ void floor_kernel(const float4 *__restrict__ aux, const float *__restrict__ rho,
                             const unsigned char *__restrict__ touched,
                             const unsigned *__restrict__ tbits, const int *d_n,
                             unsigned *d_floor)
{
    int n = *d_n;
    unsigned best = 0xffffffffu;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned alive = __float_as_uint(aux[i].w);
        unsigned hit = tbits ? (tbits[i] & alive) : (touched[i] ? alive : 0u);
        if (hit) best = min(best, f2ord(rho[i]));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) best = min(best, __shfl_xor_sync(SKID_FULL, best, o));
    if ((threadIdx.x & 31) == 0 && best != 0xffffffffu) atomicMin(d_floor, best);
}

// Pass 2: new live masks, keep flags, zeroed first-step densities.
__global__ void cut_kernel(float4 *__restrict__ aux, const float *__restrict__ rho,
                           unsigned char *__restrict__ touched, unsigned *__restrict__ tbits,
                           const int *__restrict__ sidx, const int *d_n, int cap,
                           const unsigned *d_floor, int nocut, int *__restrict__ keep, int *d_live,
                           float *__restrict__ final_rho)
{
    int n = *d_n;
    unsigned fl = *d_floor;
    float fScatDens = fl == 0xffffffffu ? 0.0f : ord2f(fl);
    int live = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        if (i >= n) { keep[i] = 0; continue; }
        float4 a = aux[i];
        unsigned alive = __float_as_uint(a.w);
        unsigned tb = tbits ? tbits[i] : 0u;
        unsigned na = alive;
        if (!nocut) {
            if (tbits) {
                if ((tb & (1u << ORIG_BIT)) == 0u && final_rho) final_rho[sidx[i]] = 0.0f;
                if (fScatDens > 0.0f) na = rho[i] >= fScatDens ? (alive & tb) : 0u;
            } else {
                na = rho[i] >= fScatDens ? alive : 0u;
            }
        }
        if (tbits) tbits[i] = 0u;
        else touched[i] = 0;
        a.w = __uint_as_float(na);
        aux[i] = a;
        keep[i] = na != 0u;
        live += __popc(na);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) live += __shfl_xor_sync(SKID_FULL, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(d_live, live);
}

// Stable compaction into the spare arrays, skipped when nothing was cut.
__global__ void compact_scat_kernel(const int *__restrict__ keep, const int *__restrict__ pos,
                                    const int *d_n, const int *d_n2,
                                    const float4 *__restrict__ spos,
                                    const float4 *__restrict__ aux, const float *__restrict__ rho,
                                    const int *__restrict__ sidx, float4 *__restrict__ spos2,
                                    float4 *__restrict__ aux2, float *__restrict__ rho2,
                                    int *__restrict__ sidx2)
{
    int n = *d_n;
    if (*d_n2 == n) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        int j = pos[i];
        spos2[j] = spos[i];
        aux2[j] = aux[i];
        rho2[j] = rho[i];
        sidx2[j] = sidx[i];
    }
}

// Copy the compacted arrays back and publish the new count.  Runs as one
// grid after the compaction, so a captured graph always reads the primary
// arrays.
__global__ void copyback_scat_kernel(int *d_n, const int *d_n2, float4 *__restrict__ spos,
                                     float4 *__restrict__ aux, float *__restrict__ rho,
                                     int *__restrict__ sidx, const float4 *__restrict__ spos2,
                                     const float4 *__restrict__ aux2,
                                     const float *__restrict__ rho2,
                                     const int *__restrict__ sidx2)
{
    int n2 = *d_n2;
    if (n2 == *d_n) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x) {
        spos[j] = spos2[j];
        aux[j] = aux2[j];
        rho[j] = rho2[j];
        sidx[j] = sidx2[j];
    }
}

__global__ void prune_flag_kernel(const float4 *__restrict__ mpos, const float4 *__restrict__ mold,
                                  const int *__restrict__ act, const int *d_nA, int cap, float3 hP,
                                  float fCvg2, int *__restrict__ keep)
{
    int n = *d_nA;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        if (i >= n) { keep[i] = 0; continue; }
        int m = act[i];
        float4 r = mpos[m], o = mold[m];
        // kd.c:752-762
        float dx = fsub(r.x, o.x), dy = fsub(r.y, o.y), dz = fsub(r.z, o.z);
        if (dx > hP.x) dx = fsub(dx, fmul(2.0f, hP.x));
        if (dx <= -hP.x) dx = fadd(dx, fmul(2.0f, hP.x));
        if (dy > hP.y) dy = fsub(dy, fmul(2.0f, hP.y));
        if (dy <= -hP.y) dy = fadd(dy, fmul(2.0f, hP.y));
        if (dz > hP.z) dz = fsub(dz, fmul(2.0f, hP.z));
        if (dz <= -hP.z) dz = fadd(dz, fmul(2.0f, hP.z));
        keep[i] = d2of(dx, dy, dz) >= fCvg2;
    }
}

__global__ void prune_compact_kernel(const int *__restrict__ keep, const int *__restrict__ pos,
                                     const int *d_nA, const int *__restrict__ act,
                                     int *__restrict__ act2, const float4 *__restrict__ mpos,
                                     float4 *__restrict__ mold)
{
    int n = *d_nA;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        int m = act[i];
        act2[pos[i]] = m;
        mold[m] = mpos[m];
    }
}

__global__ void copyback_act_kernel(int *d_nA, const int *d_nA2, int *__restrict__ act,
                                    const int *__restrict__ act2)
{
    int n2 = *d_nA2;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x)
        act[j] = act2[j];
}

__global__ void set_count_kernel(int *dst, const int *src) { *dst = *src; }

inline int grid_for(int n, int threads = 256)
{
    int b = (n + threads - 1) / threads;
    int cap = num_sms() * 8;
    if (b > cap) b = cap;
    return b < 1 ? 1 : b;
}

}  // namespace

cudaError_t scatter_aux(const float4 *spos, const float *ball2_sorted, int n, float3 L,
                        float3 boxlo, float3 boxhi, bool periodic, float4 *aux, int *d_extra,
                        cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(d_extra, 0, sizeof(int), st);
    if (e || n <= 0) return e;
    aux_kernel<<<grid_for(n), 256, 0, st>>>(spos, ball2_sorted, n, L, boxlo, boxhi,
                                            periodic ? 1 : 0, aux, d_extra);
    return cudaGetLastError();
}

cudaError_t scatter_cut(ScatState &s, bool initial, bool nocut, float *final_rho, SortScratch &ss,
                        cudaStream_t st)
{
    cudaError_t e;
    int cap = (int)s.spos.n;
    if ((e = cudaMemsetAsync(s.d_floor, 0xff, sizeof(unsigned), st))) return e;
    if ((e = cudaMemsetAsync(s.d_live, 0, sizeof(int), st))) return e;
    int g = grid_for(cap);
    floor_kernel<<<g, 256, 0, st>>>(s.saux.p, s.srho.p, s.touched.p, initial ? s.tbits.p : nullptr,
                                    s.d_nS, s.d_floor);
    cut_kernel<<<g, 256, 0, st>>>(s.saux.p, s.srho.p, s.touched.p, initial ? s.tbits.p : nullptr,
                                  s.sidx.p, s.d_nS, cap, s.d_floor, nocut ? 1 : 0, s.keep.p,
                                  s.d_live, final_rho);
    if ((e = cudaGetLastError())) return e;
    if (nocut) return cudaSuccess;
    // stable compaction of the scatterers that keep a live copy
    if ((e = scan_exclusive(s.keep.p, s.kpos.p, cap, s.d_nS2, ss, st))) return e;
    compact_scat_kernel<<<g, 256, 0, st>>>(s.keep.p, s.kpos.p, s.d_nS, s.d_nS2, s.spos.p, s.saux.p,
                                           s.srho.p, s.sidx.p, s.spos2.p, s.saux2.p, s.srho2.p,
                                           s.sidx2.p);
    copyback_scat_kernel<<<g, 256, 0, st>>>(s.d_nS, s.d_nS2, s.spos.p, s.saux.p, s.srho.p, s.sidx.p,
                                            s.spos2.p, s.saux2.p, s.srho2.p, s.sidx2.p);
    set_count_kernel<<<1, 1, 0, st>>>(s.d_nS, s.d_nS2);
    return cudaGetLastError();
}

cudaError_t mover_prune(MoverState &m, float3 period, float fCvg, SortScratch &ss, cudaStream_t st)
{
    cudaError_t e;
    int cap = (int)m.act.n;
    float3 hP = make_float3((float)(0.5 * (double)period.x), (float)(0.5 * (double)period.y),
                            (float)(0.5 * (double)period.z));
    float fCvg2 = fCvg * fCvg;
    int g = grid_for(cap);
    prune_flag_kernel<<<g, 256, 0, st>>>(m.mpos.p, m.mold.p, m.act.p, m.d_nA, cap, hP, fCvg2,
                                         m.keep.p);
    if ((e = scan_exclusive(m.keep.p, m.kpos.p, cap, m.d_nA2, ss, st))) return e;
    prune_compact_kernel<<<g, 256, 0, st>>>(m.keep.p, m.kpos.p, m.d_nA, m.act.p, m.act2.p, m.mpos.p,
                                            m.mold.p);
    copyback_act_kernel<<<g, 256, 0, st>>>(m.d_nA, m.d_nA2, m.act.p, m.act2.p);
    set_count_kernel<<<1, 1, 0, st>>>(m.d_nA, m.d_nA2);
    return cudaGetLastError();
}

}  // namespace skid
