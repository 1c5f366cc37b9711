// Adjoint (reverse-mode) kernels of the SPH density and of the group
// potential energy with respect to particle positions.  No reference
// counterpart: the reference evaluates these quantities (smooth1.c:132-276,
// grav.c:8-60) but never differentiates them.
//
// Density.  With the neighbour sets of skid_density held fixed,
//   L = sum_i w_i rho_i = sum_i sum_{j in B(i)} P_ij W(r_ij, h_i),
//   P_ij = (w_i m_j + w_j m_i) / 2,  h_i^2 = fBall2_i / 4,
// B(i) the ball of i (self included), W the M4 kernel (1/(pi h^3)) f(q).
// Differentiating each term in r_ij and in h_i (h_i = |x_i - x_K(i)|/2,
// K(i) the k-th neighbour, the one at distance^2 == fBall2_i):
//   dW/dr = (1/(pi h^5)) F(q) r,         F = f'(q)/q = -3 + 9q/4 (q<1),
//                                                      -3(2-q)^2/(4q) (q<2)
//   dW/dh = -(1/(pi h^4)) g(q),          g = 3f + q f' = 3 - 15q^2/2 + 9q^3/2 (q<1),
//                                                        3(2-q)^2 (1-q)/2 (q<2)
// so dL/dx_p gets  P F(q)/(pi h^5) (x_p - x_j)  for every pair it is an end
// of (in the frame and with the h of the ball that holds the pair), and
// H_i (x_i - x_K)/(4 h_i) at i, minus the same at K(i), with
// H_i = sum_{j in B(i)} P_ij dW/dh (r_ij, h_i).  F is the reference's move
// field profile (smooth1.c:447-459); the move field itself is minus the
// gradient of the density field rho_f(y) = sum_j m_j W(|y - x_j|, h_j) at the
// mover, i.e. the query-position adjoint with a unit cotangent, which the
// move kernel computes.
//
// Two ways to find the pairs: walk the scatterer tree again (the same walk
// as the density gather; each particle gathers both halves and needs atomics
// only for the h term of its k-th neighbour), or gather every ball's list
// once into memory (n x (k + slack) indices) and scatter from the lists.
//
// Potential energy of a group g (the pair potential of kdCellPot, grav.c:8-36,
// grav.h:11-31, on member coordinates relative to the group's reference
// point as in kdUnbind, kd.c:1338-1352):
//   E_g = -1/2 sum_{i != j} G m_i m_j psi(r_ij, eps_i + eps_j)
//   dE_g/dx_i = -G m_i sum_{j != i} m_j (psi'(r_ij)/r_ij) (x_i - x_j)
// psi'/r follows from differentiating the spline polynomials (Hernquist &
// Katz 1989): (2/e)^3 (-4/3 + 6u^2/5 - u^3/2) for u = 2r/e < 1,
// 1/(15 r^3) + (2/e)^3 (-8/3 + 3u - 6u^2/5 + u^3/6) for u < 2, -1/r^3 beyond;
// Plummer -(r^2 + e^2/4)^(-3/2).  Pair sums are FP32; the per-group energy
// total is FP64.
#include <cfloat>
#include <vector>

#include "ctx.h"

namespace skid {

namespace {

constexpr int A_WARPS = 4;
constexpr float INV_PI = 0.318309886183790671538f;

__device__ __forceinline__ float img_shift(float x, int s, float L)
{
    return s == 0 ? x : (s < 0 ? fsub(x, L) : fadd(x, L));
}

// F(q) = f'(q)/q of the M4 kernel, from q^2.
__device__ __forceinline__ float kern_F(float q2)
{
    float q = sqrtf(q2);
    if (q2 < 1.0f) return -3.0f + 2.25f * q;
    float t = 2.0f - q;
    return -0.75f * t * t / q;
}

// g(q) = 3 f(q) + q f'(q), from q^2.
__device__ __forceinline__ float kern_g(float q2)
{
    float q = sqrtf(q2);
    if (q2 < 1.0f) return 3.0f - 7.5f * q2 + 4.5f * q2 * q;
    float t = 2.0f - q;
    return 1.5f * t * t * (1.0f - q);
}

__device__ __forceinline__ void add3(float *g, float s, float x, float y, float z)
{
    g[0] += s * x;
    g[1] += s * y;
    g[2] += s * z;
}

__device__ __forceinline__ void atomic_add3(float *g, float x, float y, float z)
{
    atomicAdd(g, x);
    atomicAdd(g + 1, y);
    atomicAdd(g + 2, z);
}

// Per-particle constants of its own ball: 1/(pi h^5), -1/(pi h^4), 1/(4h).
struct Ball {
    float b, ih2, c5, c4, q4;
};

__device__ __forceinline__ Ball ball_of(float b)
{
    Ball r;
    r.b = b;
    r.ih2 = 4.0f / b;
    float ih = sqrtf(r.ih2);
    r.c4 = -INV_PI * r.ih2 * r.ih2;
    r.c5 = INV_PI * r.ih2 * r.ih2 * ih;
    r.q4 = 0.25f * ih;
    return r;
}

// The h term of particle i once H_i is complete: +c (x_i - x_K) at i, -c at K.
__device__ __forceinline__ void h_term(float *gi, float *grad, int K, float H, const Ball &bi,
                                       float kx, float ky, float kz)
{
    float c = H * bi.q4;
    add3(gi, c, kx, ky, kz);
    atomic_add3(grad + 3 * (size_t)K, -c * kx, -c * ky, -c * kz);
}

__global__ void __launch_bounds__(A_WARPS * 32)
density_adjoint_walk(TreeView t, const float *__restrict__ ball2, const float *__restrict__ wsort,
                     float3 L, float3 hL, bool per, int subShift, float *__restrict__ grad,
                     int *work, unsigned *status)
{
    __shared__ float4 cpos[A_WARPS][SKID_LEAF];
    __shared__ float4 caux[A_WARPS][SKID_LEAF];   // fBall2, 1/h^2, 1/(pi h^5), w
    __shared__ int cslot[A_WARPS][SKID_LEAF];
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
        Ball bi = ball_of(ball2[valid ? qi : base]);
        float wi = wsort[valid ? qi : base], mi = qp.w;
        // the query leaf's box (its points) and largest ball
        const float4 qlo = t.lo[t.leafBase + leaf], qhi = t.hi[t.leafBase + leaf];
        float g[3] = {0.0f, 0.0f, 0.0f};
        float H = 0.0f;
        int K = -1;
        float kx = 0.0f, ky = 0.0f, kz = 0.0f;
        int cp = 1;
        for (;;) {
            if (cp >= rootLo) {
                // the subtree's leaves one per lane against the query box, then
                // each passing leaf in order; at a leaf only candidates whose
                // distance to the query box is below max(their ball, the
                // largest query ball) can enter either half
                const int first = cp << subShift;
                bool pass = false;
                if (lane < (1 << subShift) && first + lane - t.leafBase < t.nLeaf) {
                    float4 bl = t.lo[first + lane];
                    pass = boxbox_lb(qlo, qhi, bl, t.hi[first + lane], L, per) < fmaxf(qlo.w, bl.w);
                }
                for (unsigned lm = __ballot_sync(SKID_FULL, pass); lm; lm &= lm - 1) {
                    const int node = first + __ffs(lm) - 1;
                    float4 blo = t.lo[node], bhi = t.hi[node];
                    bool want = box_lb(q, blo, bhi, L, per) < fmaxf(bi.b, blo.w);
                    if (!__any_sync(SKID_FULL, want)) continue;
                    const int cb = (node - t.leafBase) * SKID_LEAF;
                    const int cnt = min(SKID_LEAF, t.n - cb);
                    bool rel = false;
                    float4 c4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    float b = 0.0f;
                    if (lane < cnt) {
                        c4 = t.pos[cb + lane];
                        b = ball2[cb + lane];
                        rel = box_lb(make_float3(c4.x, c4.y, c4.z), qlo, qhi, L, per) < fmaxf(b, qlo.w);
                    }
                    const unsigned R = __ballot_sync(SKID_FULL, rel);
                    const int nR = __popc(R);
                    __syncwarp();
                    if (rel) {
                        const int k = __popc(R & ((1u << lane) - 1u));
                        float ih2 = 4.0f / b;
                        cpos[w][k] = c4;
                        caux[w][k] = make_float4(b, ih2, INV_PI * ih2 * ih2 * sqrtf(ih2), wsort[cb + lane]);
                        cslot[w][k] = cb + lane;
                    }
                    __syncwarp();
                    if (!want) continue;
                    int cx = img_class(q.x, blo.x, bhi.x, hL.x);
                    int cy = img_class(q.y, blo.y, bhi.y, hL.y);
                    int cz = img_class(q.z, blo.z, bhi.z, hL.z);
                    bool slow = (cx == 2) | (cy == 2) | (cz == 2);
                    float sx = img_shift(q.x, cx, L.x), sy = img_shift(q.y, cy, L.y),
                          sz = img_shift(q.z, cz, L.z);
                    for (int j = 0; j < nR; ++j) {
                        float4 cj = cpos[w][j];
                        float4 aj = caux[w][j];
                        // (ax, ay, az): x_i - x_j in i's frame; (bx, by, bz): in j's frame
                        float ax, ay, az, bx, by, bz;
                        if (slow) {
                            ax = img_dx(q.x, cj.x, L.x, hL.x);
                            ay = img_dx(q.y, cj.y, L.y, hL.y);
                            az = img_dx(q.z, cj.z, L.z, hL.z);
                            bx = -img_dx(cj.x, q.x, L.x, hL.x);
                            by = -img_dx(cj.y, q.y, L.y, hL.y);
                            bz = -img_dx(cj.z, q.z, L.z, hL.z);
                        } else {
                            ax = fsub(sx, cj.x);
                            ay = fsub(sy, cj.y);
                            az = fsub(sz, cj.z);
                            bx = -fsub(img_shift(cj.x, -cx, L.x), q.x);
                            by = -fsub(img_shift(cj.y, -cy, L.y), q.y);
                            bz = -fsub(img_shift(cj.z, -cz, L.z), q.z);
                        }
                        float dik = d2of(ax, ay, az);
                        float dki = d2of(bx, by, bz);
                        float P = 0.5f * (wi * cj.w + aj.w * mi);
                        if (dik < bi.b) {
                            float q2 = dik * bi.ih2;
                            add3(g, P * bi.c5 * kern_F(q2), ax, ay, az);
                            H += P * bi.c4 * kern_g(q2);
                        }
                        const int sj = cslot[w][j];
                        if (dik == bi.b && sj != qi) {
                            K = sj;
                            kx = ax; ky = ay; kz = az;
                        }
                        if (dki < aj.x) add3(g, P * aj.z * kern_F(dki * aj.y), bx, by, bz);
                    }
                }
            } else {
                float4 blo = t.lo[cp], bhi = t.hi[cp];
                bool want = box_lb(q, blo, bhi, L, per) < fmaxf(bi.b, blo.w);
                if (__any_sync(SKID_FULL, want)) { cp <<= 1; continue; }
            }
            cp = next_node(cp);
            if (cp == 1) break;
        }
        if (valid) {
            if (K >= 0) h_term(g, grad, K, H, bi, kx, ky, kz);
            else set_status(status, ST_BADSTATE);
            atomic_add3(grad + 3 * (size_t)qi, g[0], g[1], g[2]);
        }
    }
}

// Gather every ball's members (distance^2 <= fBall2, the kNN set with its
// ties) into rows of `cap` sorted-order indices.
__global__ void __launch_bounds__(A_WARPS * 32)
ball_lists(TreeView t, const float *__restrict__ ball2, float3 L, float3 hL, bool per, int cap,
           int *__restrict__ nbr, int *__restrict__ ncnt, int *work, unsigned *status)
{
    __shared__ float4 cpos[A_WARPS][SKID_LEAF];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
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
        int c = 0;
        int *row = nbr + (size_t)(valid ? qi : 0) * cap;
        int cp = 1;
        for (;;) {
            float4 blo = t.lo[cp], bhi = t.hi[cp];
            bool want = valid && box_lb(q, blo, bhi, L, per) <= bi;
            if (__any_sync(SKID_FULL, want)) {
                if (cp < t.leafBase) { cp <<= 1; continue; }
                int lf = cp - t.leafBase;
                if (lf < t.nLeaf) {
                    int cb = lf * SKID_LEAF;
                    int cnt = min(SKID_LEAF, t.n - cb);
                    __syncwarp();
                    if (lane < cnt) cpos[w][lane] = t.pos[cb + lane];
                    __syncwarp();
                    if (want) {
                        for (int j = 0; j < cnt; ++j) {
                            float4 cj = cpos[w][j];
                            float d = per ? d2of(img_dx(q.x, cj.x, L.x, hL.x), img_dx(q.y, cj.y, L.y, hL.y),
                                                 img_dx(q.z, cj.z, L.z, hL.z))
                                          : d2of(fsub(q.x, cj.x), fsub(q.y, cj.y), fsub(q.z, cj.z));
                            if (d <= bi) {
                                if (c < cap) row[c] = cb + j;
                                ++c;
                            }
                        }
                    }
                }
            }
            cp = next_node(cp);
            if (cp == 1) break;
        }
        if (valid) {
            if (c > cap) set_status(status, ST_OVERFLOW);
            ncnt[qi] = min(c, cap);
        }
    }
}

// Scatter form over the stored lists: each (i, j in B(i)) once, both ends.
__global__ void density_adjoint_lists(const float4 *__restrict__ pos, const float *__restrict__ ball2,
                                      const float *__restrict__ wsort, int n, float3 L, float3 hL,
                                      bool per, int cap, const int *__restrict__ nbr,
                                      const int *__restrict__ ncnt, float *__restrict__ grad,
                                      unsigned *status)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 pi = pos[i];
        Ball bi = ball_of(ball2[i]);
        float wi = wsort[i];
        float g[3] = {0.0f, 0.0f, 0.0f};
        float H = 0.0f;
        int K = -1;
        float kx = 0.0f, ky = 0.0f, kz = 0.0f;
        const int *row = nbr + (size_t)i * cap;
        int c = ncnt[i];
        for (int k = 0; k < c; ++k) {
            int j = row[k];
            float4 pj = pos[j];
            float ax, ay, az;
            if (per) {
                ax = img_dx(pi.x, pj.x, L.x, hL.x);
                ay = img_dx(pi.y, pj.y, L.y, hL.y);
                az = img_dx(pi.z, pj.z, L.z, hL.z);
            } else {
                ax = fsub(pi.x, pj.x);
                ay = fsub(pi.y, pj.y);
                az = fsub(pi.z, pj.z);
            }
            float d = d2of(ax, ay, az);
            if (d == bi.b && j != i) {
                K = j;
                kx = ax; ky = ay; kz = az;
            }
            if (!(d < bi.b)) continue;
            float P = 0.5f * (wi * pj.w + wsort[j] * pi.w);
            float q2 = d * bi.ih2;
            float s = P * bi.c5 * kern_F(q2);
            add3(g, s, ax, ay, az);
            if (j != i) atomic_add3(grad + 3 * (size_t)j, -s * ax, -s * ay, -s * az);
            H += P * bi.c4 * kern_g(q2);
        }
        if (K >= 0) h_term(g, grad, K, H, bi, kx, ky, kz);
        else set_status(status, ST_BADSTATE);
        atomic_add3(grad + 3 * (size_t)i, g[0], g[1], g[2]);
    }
}

__global__ void gather_w(const int *__restrict__ sidx, const float *__restrict__ w_io, int n,
                         float *__restrict__ w_sorted)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w_sorted[i] = w_io[sidx[i]];
}

__global__ void scatter_grad(const int *__restrict__ sidx, const float *__restrict__ g_sorted, int n,
                             float *__restrict__ g_io)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int o = sidx[i];
        g_io[3 * (size_t)o] = g_sorted[3 * (size_t)i];
        g_io[3 * (size_t)o + 1] = g_sorted[3 * (size_t)i + 1];
        g_io[3 * (size_t)o + 2] = g_sorted[3 * (size_t)i + 2];
    }
}

// ---- group potential energy ----

constexpr int PA_TILE = 128;

// psi(r, e) as kdCellPot evaluates it (grav.h:11-31) and psi'(r)/r.
// Beyond the softening (r >= 2h, certain once d2 clears (2h)^2 by the margin
// below) and for Plummer softening, psi comes from the hardware reciprocal
// square root (2 ulp).
__device__ __forceinline__ void pair_psi(float d2, float twoh, int plummer, float &psi, float &gr)
{
    if (plummer || d2 >= twoh * twoh * 1.000001f) {
        float t = rsqrtf(plummer ? d2 + 0.25f * twoh * twoh : d2);
        psi = t;
        gr = -t * t * t;
        return;
    }
    float r = sqrtf(d2);
    if (r < twoh) {
        float dih = 2.0f / twoh;
        float u = r * dih;
        float u2 = u * u;
        float d3 = dih * dih * dih;
        if (u < 1.0f) {
            psi = dih * (1.4f - (2.0f / 3.0f) * u2 + 0.3f * u2 * u2 - 0.1f * u2 * u2 * u);
            gr = d3 * (-4.0f / 3.0f + 1.2f * u2 - 0.5f * u2 * u);
        } else {
            psi = -(1.0f / 15.0f) / r +
                  dih * (1.6f - (4.0f / 3.0f) * u2 + u2 * u - 0.3f * u2 * u2 + (1.0f / 30.0f) * u2 * u2 * u);
            gr = (1.0f / 15.0f) / (d2 * r) + d3 * (-8.0f / 3.0f + 3.0f * u - 1.2f * u2 + (1.0f / 6.0f) * u2 * u);
        }
        return;
    }
    psi = 1.0f / r;
    gr = -psi / d2;
}

__device__ __forceinline__ float wrap_rel(float d, float h)
{
    if (d > h) d = fsub(d, fmul(2.0f, h));
    if (d <= -h) d = fadd(d, fmul(2.0f, h));
    return d;
}

struct PotAdjArgs {
    const int2 *items;          // (selection slot, tile)
    int nitems;
    const int *gsel;            // group id per slot
    const float *v;             // cotangent per slot (may be null: no gradient)
    const int *gstart, *gcount, *members;
    const float4 *pos4, *vel4;  // (x, y, z, m), (vx, vy, vz, soft)
    const skid_group *rec;
    float3 hP;
    float G;
    int plummer;
    double *E;                  // per slot
    float *grad;                // 3n by iOrder (zeroed) or null
};

// One (selection slot, row tile) per block iteration: PA_TILE / 2 threads,
// each with rows t and t + PA_TILE / 2, over every column tile of the group.
constexpr int PA_THREADS = PA_TILE / 2;

struct PaRow {
    float3 r;
    float e, m;
    int io;
    bool v;
    float phi, phic, gx, gy, gz;   // Kahan-compensated sum_j m_j psi_ij; sum_j m_j psi'/r (x_i - x_j)
};

__device__ __forceinline__ void pa_row_init(PaRow &w, const PotAdjArgs &a, int s, int n, int i,
                                            const float *rel)
{
    w.v = i < n;
    w.io = w.v ? a.members[s + i] : 0;
    float4 p = a.pos4[w.io];
    w.m = p.w;
    w.e = a.vel4[w.io].w;
    w.r = make_float3(wrap_rel(fsub(p.x, rel[0]), a.hP.x), wrap_rel(fsub(p.y, rel[1]), a.hP.y),
                      wrap_rel(fsub(p.z, rel[2]), a.hP.z));
    w.phi = w.phic = w.gx = w.gy = w.gz = 0.0f;
}

__device__ __forceinline__ void pa_row_add(PaRow &w, float4 rj, float ej, int plummer)
{
    float dx = w.r.x - rj.x, dy = w.r.y - rj.y, dz = w.r.z - rj.z;
    float psi, gr;
    pair_psi(dx * dx + dy * dy + dz * dz, w.e + ej, plummer, psi, gr);
    float y = rj.w * psi - w.phic;
    float tt = w.phi + y;
    w.phic = (tt - w.phi) - y;
    w.phi = tt;
    float c = rj.w * gr;
    w.gx += c * dx;
    w.gy += c * dy;
    w.gz += c * dz;
}

__global__ void __launch_bounds__(PA_THREADS) potential_adjoint_kernel(PotAdjArgs a)
{
    __shared__ float4 sr[PA_TILE];
    __shared__ float ss[PA_TILE];
    __shared__ double red[PA_THREADS / 32];
    const int tid = threadIdx.x;
    for (int it = blockIdx.x; it < a.nitems; it += gridDim.x) {
        int2 item = a.items[it];
        int slot = item.x;
        int g = a.gsel[slot];
        int s = a.gstart[g], n = a.gcount[g];
        const float *rel = a.rec[g].rel;
        const int i0 = item.y * PA_TILE + tid, i1 = i0 + PA_THREADS;
        PaRow r0, r1;
        pa_row_init(r0, a, s, n, i0, rel);
        pa_row_init(r1, a, s, n, i1, rel);
        for (int jb = 0; jb < n; jb += PA_TILE) {
            __syncthreads();
            for (int c = tid; c < PA_TILE; c += PA_THREADS) {
                int j = jb + c;
                if (j < n) {
                    int jo = a.members[s + j];
                    float4 q = a.pos4[jo];
                    sr[c] = make_float4(wrap_rel(fsub(q.x, rel[0]), a.hP.x), wrap_rel(fsub(q.y, rel[1]), a.hP.y),
                                        wrap_rel(fsub(q.z, rel[2]), a.hP.z), q.w);
                    ss[c] = a.vel4[jo].w;
                }
            }
            __syncthreads();
            const int cnt = min(PA_TILE, n - jb);
            for (int k = 0; k < cnt; ++k) {
                const float4 rj = sr[k];
                const float ej = ss[k];
                if (r0.v && jb + k != i0) pa_row_add(r0, rj, ej, a.plummer);
                if (r1.v && jb + k != i1) pa_row_add(r1, rj, ej, a.plummer);
            }
        }
        // E contribution -1/2 G m_i phi_i, summed over the tile in FP64
        double e = (r0.v ? -0.5 * (double)a.G * (double)r0.m * (double)r0.phi : 0.0) +
                   (r1.v ? -0.5 * (double)a.G * (double)r1.m * (double)r1.phi : 0.0);
        for (int o = 16; o; o >>= 1) e += __shfl_xor_sync(SKID_FULL, e, o);
        if ((tid & 31) == 0) red[tid >> 5] = e;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int k = 0; k < PA_THREADS / 32; ++k) t += red[k];
            atomicAdd(a.E + slot, t);
        }
        if (a.grad) {
            const PaRow *rows[2] = {&r0, &r1};
            for (int q = 0; q < 2; ++q) {
                const PaRow &w = *rows[q];
                if (!w.v) continue;
                float c = -a.G * w.m * a.v[slot];
                float *o = a.grad + 3 * (size_t)w.io;
                o[0] = c * w.gx;
                o[1] = c * w.gy;
                o[2] = c * w.gz;
            }
        }
    }
}

}  // namespace

cudaError_t density_adjoint(const Tree &t, const float *ball2_sorted, const int *sidx, const float *w_io,
                            int n_io, float3 L, bool per, int mode, int k, AdjointState &A,
                            int *d_work, unsigned *d_status, cudaStream_t st)
{
    cudaError_t e;
    int ns = t.n;
    size_t m = ns > 0 ? ns : 1;
    if ((e = dalloc(A.w, m)) || (e = dalloc(A.g, 3 * m)) || (e = dalloc(A.out, 3 * (size_t)(n_io > 0 ? n_io : 1))))
        return e;
    if ((e = cudaMemsetAsync(A.g.p, 0, 3 * m * sizeof(float), st))) return e;
    if ((e = cudaMemsetAsync(A.out.p, 0, 3 * (size_t)(n_io > 0 ? n_io : 1) * sizeof(float), st))) return e;
    if (ns <= 0) return cudaSuccess;
    gather_w<<<grid_for(ns), 256, 0, st>>>(sidx, w_io, ns, A.w.p); note_launch();
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    int need = (t.nLeaf + A_WARPS - 1) / A_WARPS;
    if (mode == 2) {
        // store the lists only while they take at most a quarter of the free memory
        size_t fr = 0, tot = 0;
        size_t bytes = m * (size_t)(k + 16 + 1) * sizeof(int);
        mode = (A.lists || (cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes <= fr / 4)) ? 1 : 0;
    }
    if (mode == 0) {
        if ((e = cudaMemsetAsync(d_work, 0, sizeof(int), st))) return e;
        int perSM = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, density_adjoint_walk, A_WARPS * 32, 0);
        int blocks = num_sms() * (perSM > 0 ? perSM : 1);
        if (blocks > need) blocks = need;
        int subShift = 0;
        while (subShift < 5 && (2 << subShift) <= t.leafBase) ++subShift;
        density_adjoint_walk<<<blocks, A_WARPS * 32, 0, st>>>(t.view(), ball2_sorted, A.w.p, L, hL, per,
                                                             subShift, A.g.p, d_work, d_status); note_launch();
    } else {
        if (!A.lists) {
            A.cap = k + 16;
            if ((e = dalloc(A.nbr, m * (size_t)A.cap)) || (e = dalloc(A.ncnt, m))) return e;
            if ((e = cudaMemsetAsync(d_work, 0, sizeof(int), st))) return e;
            int perSM = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, ball_lists, A_WARPS * 32, 0);
            int blocks = num_sms() * (perSM > 0 ? perSM : 1);
            if (blocks > need) blocks = need;
            ball_lists<<<blocks, A_WARPS * 32, 0, st>>>(t.view(), ball2_sorted, L, hL, per, A.cap,
                                                       A.nbr.p, A.ncnt.p, d_work, d_status); note_launch();
            A.lists = true;
        }
        density_adjoint_lists<<<grid_for(ns, 128), 128, 0, st>>>(t.pos.p, ball2_sorted, A.w.p, ns, L, hL,
                                                                per, A.cap, A.nbr.p, A.ncnt.p, A.g.p,
                                                                d_status); note_launch();
    }
    scatter_grad<<<grid_for(ns), 256, 0, st>>>(sidx, A.g.p, ns, A.out.p); note_launch();
    return cudaGetLastError();
}

cudaError_t potential_adjoint(const GroupState &G, const float4 *pos4, const float4 *vel4, int n,
                              float3 period, float Gc, int plummer, int nSel, const int *h_sel,
                              const float *h_v, bool want_grad, AdjointState &A, cudaStream_t st)
{
    cudaError_t e;
    std::vector<int> counts(G.nGroup);
    if ((e = cudaMemcpyAsync(counts.data(), G.count.p, G.nGroup * sizeof(int), cudaMemcpyDeviceToHost, st)))
        return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    std::vector<int2> items;
    for (int s = 0; s < nSel; ++s) {
        int c = counts[h_sel[s]];
        for (int t = 0; t * PA_TILE < c; ++t) items.push_back(make_int2(s, t));
    }
    size_t ni = items.size();
    if ((e = dalloc(A.items, ni > 0 ? ni : 1)) || (e = dalloc(A.gsel, nSel > 0 ? nSel : 1)) ||
        (e = dalloc(A.v, nSel > 0 ? nSel : 1)) || (e = dalloc(A.E, nSel > 0 ? nSel : 1)) ||
        (e = dalloc(A.out, 3 * (size_t)(n > 0 ? n : 1))))
        return e;
    if (ni && (e = cudaMemcpyAsync(A.items.p, items.data(), ni * sizeof(int2), cudaMemcpyHostToDevice, st)))
        return e;
    if (nSel) {
        if ((e = cudaMemcpyAsync(A.gsel.p, h_sel, nSel * sizeof(int), cudaMemcpyHostToDevice, st))) return e;
        if (h_v && (e = cudaMemcpyAsync(A.v.p, h_v, nSel * sizeof(float), cudaMemcpyHostToDevice, st)))
            return e;
        if ((e = cudaMemsetAsync(A.E.p, 0, nSel * sizeof(double), st))) return e;
    }
    if ((e = cudaMemsetAsync(A.out.p, 0, 3 * (size_t)(n > 0 ? n : 1) * sizeof(float), st))) return e;
    if (!ni) return cudaSuccess;
    PotAdjArgs a;
    a.items = A.items.p;
    a.nitems = (int)ni;
    a.gsel = A.gsel.p;
    a.v = A.v.p;
    a.gstart = G.start.p;
    a.gcount = G.count.p;
    a.members = G.members.p;
    a.pos4 = pos4;
    a.vel4 = vel4;
    a.rec = G.rec.p;
    a.hP = make_float3((float)(0.5 * (double)period.x), (float)(0.5 * (double)period.y),
                       (float)(0.5 * (double)period.z));
    a.G = Gc;
    a.plummer = plummer;
    a.E = A.E.p;
    a.grad = want_grad ? A.out.p : nullptr;
    int blocks = (int)(ni < (size_t)num_sms() * 32 ? ni : (size_t)num_sms() * 32);
    potential_adjoint_kernel<<<blocks, PA_THREADS, 0, st>>>(a); note_launch();
    return cudaGetLastError();
}

}  // namespace skid
