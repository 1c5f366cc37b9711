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
// Kernels: scoop lists (one thread per group walks the tree of ungrouped
// particles), the all-pairs potential (one block per 128-member tile), and
// the removal loop (one block per group, block-wide arg-max with
// first-index ties).
#include <cfloat>

#include "ctx.h"

namespace skid {

namespace {

constexpr int POT_TILE = 128;
constexpr int RM_THREADS = 256;
// Groups up to this size evaluate E exactly as the reference does (FP64
// expression rounded to float, kd.c:1396-1399), so equal-energy members are
// ordered by the reference's own rounding; larger groups use FP32 (GB300's
// FP64 rate is a small fraction of its FP32 rate).
constexpr int EXACT_E_MAX = 1024;

__device__ __forceinline__ float spline_pot(float d2, float twoh, int plummer)
{
    if (plummer) return 1.0f / sqrtf(d2 + 0.25f * twoh * twoh);
    float r = sqrtf(d2);
    if (r < twoh) {
        float dih = 2.0f / twoh;
        float u = r * dih;
        float u2 = u * u;
        if (u < 1.0f) {
            return dih * (1.4f - (2.0f / 3.0f) * u2 + 0.3f * u2 * u2 - 0.1f * u2 * u2 * u);
        }
        return -(1.0f / 15.0f) / r +
               dih * (1.6f - (4.0f / 3.0f) * u2 + u2 * u - 0.3f * u2 * u2 + (1.0f / 30.0f) * u2 * u2 * u);
    }
    return 1.0f / r;
}

__device__ __forceinline__ float wrap_h(float d, float h)
{
    // kd.c:1345-1350: if (dx > hx) dx -= 2*hx; if (dx <= -hx) dx += 2*hx
    if (d > h) d = fsub(d, fmul(2.0f, h));
    if (d <= -h) d = fadd(d, fmul(2.0f, h));
    return d;
}

// Fixed-point quantum of a float term (scale = 2^S, exact multiply).
__device__ __forceinline__ long long fx(float t, float scale) { return __float2ll_rn(t * scale); }

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
    for (int g = blockIdx.x * blockDim.x + threadIdx.x + 1; g < ng; g += gridDim.x * blockDim.x) {
        int c = 0;
        int n = gcount[g];
        if (n > 0 && n < nmax && t.n > 0) {
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

__global__ void pot_items(const int *__restrict__ gcount, int ng, int nmax,
                          const int *__restrict__ ioff, int2 *__restrict__ items)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x + 1; g < ng; g += gridDim.x * blockDim.x) {
        int n = gcount[g];
        if (n <= 0 || n >= nmax) continue;
        int nt = (n + POT_TILE - 1) / POT_TILE;
        for (int t = 0; t < nt; ++t) items[ioff[g] + t] = make_int2(g, t);
    }
}

__global__ void pot_ntiles(const int *__restrict__ gcount, int ng, int nmax, int *__restrict__ nt)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int n = gcount[g];
        nt[g] = (g > 0 && n > 0 && n < nmax) ? (n + POT_TILE - 1) / POT_TILE : 0;
    }
}

__global__ void __launch_bounds__(POT_TILE)
pot_kernel(const int2 *__restrict__ items, const int *d_nitems, const int *__restrict__ gstart,
           const int *__restrict__ gcount, const float4 *__restrict__ qr,
           const float4 *__restrict__ qv, const int *__restrict__ soff,
           const int *__restrict__ scnt, const float4 *__restrict__ slist,
           const float *__restrict__ ssoft, float G, int plummer, float scale,
           long long *__restrict__ pot)
{
    __shared__ float4 sr[POT_TILE];
    __shared__ float ss[POT_TILE];
    int nitems = *d_nitems;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        int2 w = items[it];
        int g = w.x;
        int s = gstart[g], n = gcount[g];
        int i = w.y * POT_TILE + threadIdx.x;
        bool valid = i < n;
        float4 ri = valid ? qr[s + i] : make_float4(0, 0, 0, 0);
        float ei = valid ? qv[s + i].w : 0.0f;
        long long acc = 0;
        for (int jb = 0; jb < n; jb += POT_TILE) {
            __syncthreads();
            int j = jb + threadIdx.x;
            if (j < n) {
                sr[threadIdx.x] = qr[s + j];
                ss[threadIdx.x] = qv[s + j].w;
            }
            __syncthreads();
            int cnt = min(POT_TILE, n - jb);
            for (int k = 0; k < cnt; ++k) {
                float4 rj = sr[k];
                float d2 = d2of(fsub(ri.x, rj.x), fsub(ri.y, rj.y), fsub(ri.z, rj.z));
                float dir = spline_pot(d2, fadd(ei, ss[k]), plummer);
                float term = fmul(fmul(G, rj.w), dir);
                acc += (jb + k != i) ? fx(term, scale) : 0ll;
            }
        }
        // kdAddScoopPot: grav.c:112-127
        int so = soff[g], sc = scnt[g];
        for (int jb = 0; jb < sc; jb += POT_TILE) {
            __syncthreads();
            int j = jb + threadIdx.x;
            if (j < sc) {
                sr[threadIdx.x] = slist[so + j];
                ss[threadIdx.x] = ssoft[so + j];
            }
            __syncthreads();
            int cnt = min(POT_TILE, sc - jb);
            for (int k = 0; k < cnt; ++k) {
                float4 rj = sr[k];
                float d2 = d2of(fsub(rj.x, ri.x), fsub(rj.y, ri.y), fsub(rj.z, ri.z));
                float dir = spline_pot(d2, fadd(ss[k], ei), plummer);
                acc += fx(fmul(fmul(G, rj.w), dir), scale);
            }
        }
        if (valid) pot[s + i] = acc;
    }
}

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

struct RemoveArgs {
    const int *gstart, *gcount;
    int ng, nmax;
    float4 *qr, *qv;
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
};

__global__ void __launch_bounds__(RM_THREADS) remove_kernel(RemoveArgs A)
{
    __shared__ ArgRed smax[RM_THREADS / 32], smin[RM_THREADS / 32];
    __shared__ float4 s_r;      // removed particle (relative position, mass)
    __shared__ float s_eps;
    __shared__ float s_cm[6];   // rcm, vcm as floats
    __shared__ int s_n, s_go, s_have, s_imin;
    __shared__ double d_cm[6], d_mass;
    int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int g = blockIdx.x + 1; g < A.ng; g += gridDim.x) {
        int s = A.gstart[g], n0 = A.gcount[g];
        if (n0 <= 0 || n0 >= A.nmax) continue;
        float4 *qr = A.qr + s;
        float4 *qv = A.qv + s;
        int *qid = A.qid + s;
        long long *pot = A.pot + s;
        // centre of mass and velocity (kd.c:1360-1375), FP64 sums of float products
        double m = 0.0, c[6] = {0, 0, 0, 0, 0, 0};
        for (int i = tid; i < n0; i += RM_THREADS) {
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
        if (tid == 0) { d_mass = 0.0; for (int d = 0; d < 6; ++d) d_cm[d] = 0.0; }
        __syncthreads();
        if (lane == 0) {
            atomicAdd(&d_mass, m);
            for (int d = 0; d < 6; ++d) atomicAdd(&d_cm[d], c[d]);
        }
        __syncthreads();
        if (tid == 0) {
            for (int d = 0; d < 6; ++d) {
                d_cm[d] /= d_mass;
                s_cm[d] = (float)d_cm[d];
            }
            s_n = n0;
            s_have = 0;
            s_go = 1;
        }
        __syncthreads();
        int nrem = 0;
        const bool exact = n0 <= EXACT_E_MAX;
        const double opz_d = 1.0 + (double)A.z;
        const double inv_d = 1.0 / (double)A.scale;
        while (true) {
            int n = s_n;
            bool have = s_have != 0;
            float4 rs = s_r;
            float es = s_eps;
            float cm0 = s_cm[0], cm1 = s_cm[1], cm2 = s_cm[2];
            float vm0 = s_cm[3], vm1 = s_cm[4], vm2 = s_cm[5];
            double dc0 = d_cm[0], dc1 = d_cm[1], dc2 = d_cm[2];
            double dv0m = d_cm[3], dv1m = d_cm[4], dv2m = d_cm[5];
            ArgRed mx{-FLT_MAX, 0x7fffffff}, mn{FLT_MAX, 0x7fffffff};
            for (int i = tid; i < n; i += RM_THREADS) {
                float4 r = qr[i], v = qv[i];
                long long p = pot[i];
                if (have && A.subpot) {
                    // kdSubPot (grav.c:44-59)
                    float d2 = d2of(fsub(rs.x, r.x), fsub(rs.y, r.y), fsub(rs.z, r.z));
                    float dir = spline_pot(d2, fadd(es, v.w), A.plummer);
                    p -= fx(fmul(fmul(A.G, rs.w), dir), A.scale);
                    pot[i] = p;
                }
                float E;
                if (exact) {
                    double fs = A.fShift, fc = A.fCosmo;
                    float dv0 = (float)(fs * ((double)v.x - dv0m) + fc * ((double)r.x - dc0));
                    float dv1 = (float)(fs * ((double)v.y - dv1m) + fc * ((double)r.y - dc1));
                    float dv2 = (float)(fs * ((double)v.z - dv2m) + fc * ((double)r.z - dc2));
                    float dd = fadd(fadd(fmul(dv0, dv0), fmul(dv1, dv1)), fmul(dv2, dv2));
                    E = (float)(0.5 * (double)dd - ((double)p * inv_d) * opz_d);
                } else {
                    float dv0 = A.fShift * (v.x - vm0) + A.fCosmo * (r.x - cm0);
                    float dv1 = A.fShift * (v.y - vm1) + A.fCosmo * (r.y - cm1);
                    float dv2 = A.fShift * (v.z - vm2) + A.fCosmo * (r.z - cm2);
                    float dd = fadd(fadd(fmul(dv0, dv0), fmul(dv1, dv1)), fmul(dv2, dv2));
                    E = 0.5f * dd - (__ll2float_rn(p) * A.inv_scale) * A.opz;
                }
                if (E > mx.v) { mx.v = E; mx.i = i; }
                if (E < mn.v) { mn.v = E; mn.i = i; }
            }
            mx = warp_argmax(mx);
            mn = warp_argmin(mn);
            if (lane == 0) { smax[w] = mx; smin[w] = mn; }
            __syncthreads();
            if (tid == 0) {
                ArgRed a = smax[0], b = smin[0];
                for (int k = 1; k < RM_THREADS / 32; ++k) {
                    ArgRed x = smax[k], y = smin[k];
                    if (x.v > a.v || (x.v == a.v && x.i < a.i)) a = x;
                    if (y.v < b.v || (y.v == b.v && y.i < b.i)) b = y;
                }
                // kd.c:1389-1409: fTotBig starts at -1, fTotMin at 1
                s_imin = b.v < 1.0f ? b.i : 0;
                if (!(a.v >= 0.0f) || A.nounbind || n == 0) {
                    s_go = 0;
                } else {
                    int ib = a.i;
                    float4 r = qr[ib], v = qv[ib];
                    A.grp[qid[ib]] = 0;
                    ++nrem;
                    int nn = n - 1;
                    if (nn == 0) {
                        d_mass = 0.0;
                        for (int d = 3; d < 6; ++d) d_cm[d] = 0.0;
                        s_go = 0;
                    } else {
                        d_mass -= r.w;
                        double f = (double)r.w / d_mass;
                        d_cm[0] += f * (d_cm[0] - r.x);
                        d_cm[1] += f * (d_cm[1] - r.y);
                        d_cm[2] += f * (d_cm[2] - r.z);
                        d_cm[3] += f * (d_cm[3] - v.x);
                        d_cm[4] += f * (d_cm[4] - v.y);
                        d_cm[5] += f * (d_cm[5] - v.z);
                        for (int d = 0; d < 6; ++d) s_cm[d] = (float)d_cm[d];
                        // swap with the last member (kd.c:1435-1440)
                        float4 rl = qr[nn], vl = qv[nn];
                        int il = qid[nn], ir = qid[ib];
                        long long pl = pot[nn], pb = pot[ib];
                        qr[ib] = rl; qv[ib] = vl; qid[ib] = il; pot[ib] = pl;
                        qr[nn] = r; qv[nn] = v; qid[nn] = ir; pot[nn] = pb;
                        s_r = r;
                        s_eps = v.w;
                        s_have = 1;
                    }
                    s_n = nn;
                }
            }
            __syncthreads();
            if (!s_go) break;
        }
        if (tid == 0) {
            skid_group r = A.rec[g];
            int n = s_n;
            r.nMembers = n;
            r.fMass = (float)d_mass;
            r.vcm[0] = (float)d_cm[3];
            r.vcm[1] = (float)d_cm[4];
            r.vcm[2] = (float)d_cm[5];
            float4 rb = qr[s_imin];
            float hx = A.hP.x;   // kd.c:1452-1456 wraps every axis with hx
            r.rBound[0] = wrap_h(fadd(rb.x, r.rel[0]), hx);
            r.rBound[1] = wrap_h(fadd(rb.y, r.rel[1]), hx);
            r.rBound[2] = wrap_h(fadd(rb.z, r.rel[2]), hx);
            A.rec[g] = r;
            if (nrem) atomicAdd(A.d_unbound, nrem);
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t unbind_run(GroupState &G, const int *gof, int nslots, const float4 *pos4,
                       const float4 *vel4, Tree &ut, const UnbindParams &P, int *grp,
                       int *d_unbound, SortScratch &ss, UnbindScratch &U, cudaStream_t st)
{
    cudaError_t e;
    int ng = G.nGroup;
    if ((e = dalloc(U.qr, nslots)) || (e = dalloc(U.qv, nslots)) || (e = dalloc(U.qid, nslots)) ||
        (e = dalloc(U.pot, nslots)) || (e = dalloc(U.scnt, ng)) || (e = dalloc(U.soff, ng + 1)) ||
        (e = dalloc(U.nt, ng)) || (e = dalloc(U.toff, ng + 1)) || (e = dalloc(U.cnt, 4)))
        return e;
    float3 hP = make_float3((float)(0.5 * (double)P.period.x), (float)(0.5 * (double)P.period.y),
                            (float)(0.5 * (double)P.period.z));
    prep_members<<<grid_for(nslots), 256, 0, st>>>(G.members.p, gof, nslots, pos4, vel4, G.rec.p,
                                                   hP, U.qr.p, U.qv.p); skid::note_launch();
    if ((e = cudaMemcpyAsync(U.qid.p, G.members.p, nslots * sizeof(int), cudaMemcpyDeviceToDevice,
                             st)))
        return e;
    // scoop lists
    float fBall2 = P.fScoop * P.fScoop;
    float3 hL = make_float3(0.5f * P.period.x, 0.5f * P.period.y, 0.5f * P.period.z);
    scoop_kernel<<<grid_for(ng), 256, 0, st>>>(ut.view(), U.usoft.p, G.rec.p, G.count.p, ng, P.nmax,
                                              fBall2, P.period, hL, P.per, 0, U.scnt.p, nullptr,
                                              nullptr, nullptr); skid::note_launch();
    if ((e = scan_exclusive(U.scnt.p, U.soff.p, ng, U.cnt.p, ss, st))) return e;
    int nscoop = 0;
    if ((e = cudaMemcpyAsync(&nscoop, U.cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    if ((e = dalloc(U.slist, nscoop > 0 ? nscoop : 1)) || (e = dalloc(U.ssoft, nscoop > 0 ? nscoop : 1)))
        return e;
    if (nscoop > 0)
        scoop_kernel<<<grid_for(ng), 256, 0, st>>>(ut.view(), U.usoft.p, G.rec.p, G.count.p, ng,
                                                  P.nmax, fBall2, P.period, hL, P.per, 1, U.scnt.p,
                                                  U.soff.p, U.slist.p, U.ssoft.p); skid::note_launch();
    // potential work items (group, tile)
    pot_ntiles<<<grid_for(ng), 256, 0, st>>>(G.count.p, ng, P.nmax, U.nt.p); skid::note_launch();
    if ((e = scan_exclusive(U.nt.p, U.toff.p, ng, U.cnt.p + 1, ss, st))) return e;
    int nitems = 0;
    if ((e = cudaMemcpyAsync(&nitems, U.cnt.p + 1, sizeof(int), cudaMemcpyDeviceToHost, st)))
        return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    if ((e = dalloc(U.items, nitems > 0 ? nitems : 1))) return e;
    if (nitems > 0) {
        pot_items<<<grid_for(ng), 256, 0, st>>>(G.count.p, ng, P.nmax, U.toff.p, U.items.p); skid::note_launch();
        int blocks = nitems < num_sms() * 16 ? nitems : num_sms() * 16;
        pot_kernel<<<blocks, POT_TILE, 0, st>>>(U.items.p, U.cnt.p + 1, G.start.p, G.count.p, U.qr.p,
                                                U.qv.p, U.soff.p, U.scnt.p, U.slist.p, U.ssoft.p,
                                                P.G, P.plummer, P.scale, U.pot.p); skid::note_launch();
    }
    // removal loop, one block per group
    RemoveArgs A;
    A.gstart = G.start.p;
    A.gcount = G.count.p;
    A.ng = ng;
    A.nmax = P.nmax;
    A.qr = U.qr.p;
    A.qv = U.qv.p;
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
    if ((e = cudaMemsetAsync(d_unbound, 0, sizeof(int), st))) return e;
    int blocks = ng - 1 < num_sms() * 8 ? ng - 1 : num_sms() * 8;
    if (blocks > 0) remove_kernel<<<blocks, RM_THREADS, 0, st>>>(A); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
