// Scatterer copies and mover bookkeeping for the move phase.
//
//  - copies: every scatterer plus each periodic image whose distance to the
//    box is below fBall2 (the replica scatterers of smooth1.c:283-332, same
//    float arithmetic as INTERSECTNP, kd.h:102-119).  A copy carries its own
//    position x_c = fl(x + s L), so the move-field gather is a plain
//    (non-periodic) ball test from the copy, like smBallGather
//    (smooth1.c:338-384).  Slots hold
//        cpos  = (x_c, y_c, z_c, fBall2)
//        ccoef = (ih2, fNorm*m, rho, iOrder | original-bit)
//    with ih2 = 4/fBall2 and fNorm = M_1_PI ih2^2 sqrt(ih2) m rounded like
//    smooth1.c:447-448.
//  - cut: the heuristic scatterer removal (smooth1.c:460-470, 387-405,
//    509-513).  fScatDens = min density over copies that reached an active
//    mover; copies below it go.  On the first step (dark-only input or -fic)
//    copies that reached no mover count as density 0.  A copy cut is marked
//    dead in its slot (empty ball, density -inf); the survivors are compacted
//    in slot order, which keeps them Hilbert-sorted, at the last step of each
//    outer iteration (and after every single step), followed by a refit.
//  - prune: kdPruneInactive (kd.c:735-793), stable, then the active movers
//    are re-sorted by the Hilbert key of their current positions so that each
//    warp's movers stay close together as the active set thins out.
#include <cfloat>
#include <cstring>

#include "internal.h"

namespace skid {

namespace {

constexpr unsigned ORIG_FLAG = 0x80000000u;

__device__ __forceinline__ unsigned image_mask(float4 p, float b, float3 L, float3 blo, float3 bhi)
{
    unsigned m = 0;
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
    return m;
}

__global__ void copy_count_kernel(const float4 *__restrict__ spos, const float *__restrict__ ball2,
                                  int n, float3 L, float3 blo, float3 bhi, int periodic,
                                  unsigned *__restrict__ masks, int *__restrict__ counts)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned m = periodic ? image_mask(spos[i], ball2[i], L, blo, bhi) : 0u;
        masks[i] = m;
        counts[i] = 1 + __popc(m);
    }
}

__global__ void copy_write_kernel(const float4 *__restrict__ spos, const float *__restrict__ ball2,
                                  const float *__restrict__ rho, const int *__restrict__ sidx,
                                  const unsigned *__restrict__ masks, const int *__restrict__ off,
                                  int n, float3 L, float4 *__restrict__ cpos,
                                  float4 *__restrict__ ccoef)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = spos[i];
        float b = ball2[i];
        float ih2 = (float)(4.0 / (double)b);
        double dih2 = ih2;
        float fnm = (float)(M_1_PI * dih2 * dih2 * sqrt(dih2) * (double)p.w);
        float r = rho[i];
        unsigned io = (unsigned)sidx[i];
        int o = off[i];
        cpos[o] = make_float4(p.x, p.y, p.z, b);
        ccoef[o] = make_float4(ih2, fnm, r, __uint_as_float(io | ORIG_FLAG));
        unsigned m = masks[i];
        int k = 1;
        while (m) {
            int bit = __ffs(m) - 1;
            m &= m - 1;
            int ix = bit / 9 - 1, iy = (bit / 3) % 3 - 1, iz = bit % 3 - 1;
            float x = fadd(p.x, fmul((float)ix, L.x));
            float y = fadd(p.y, fmul((float)iy, L.y));
            float z = fadd(p.z, fmul((float)iz, L.z));
            cpos[o + k] = make_float4(x, y, z, b);
            ccoef[o + k] = make_float4(ih2, fnm, r, __uint_as_float(io));
            ++k;
        }
    }
}

__global__ void copy_keys_kernel(const float4 *__restrict__ cpos, int n, float3 lo, float3 inv, int hil,
                                 uint64_t *keys, uint32_t *vals)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = cpos[i];
        keys[i] = curve63(make_float3(q.x, q.y, q.z), lo, inv, hil != 0);
        vals[i] = (uint32_t)i;
    }
}

__global__ void copy_permute_kernel(const uint32_t *__restrict__ perm, int n,
                                    const float4 *__restrict__ a, const float4 *__restrict__ b,
                                    float4 *__restrict__ a2, float4 *__restrict__ b2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t j = perm[i];
        a2[i] = a[j];
        b2[i] = b[j];
    }
}

// ---- the cut, in tiles of CT_TILE slots: keep flags and per-tile counts,
// then each tile compacts itself from the counts before it ----
// A tile is CT_TILE slots for one block; warp w owns the CT_ITEMS x 32
// consecutive slots from w * CT_WSPAN, read 32 at a time (coalesced), with
// its in-tile offsets from ballots.
constexpr int CT_THREADS = 256;
constexpr int CT_ITEMS = 16;
constexpr int CT_TILE = CT_THREADS * CT_ITEMS;   // matches the blk sizing (4096)
constexpr int CT_WSPAN = CT_ITEMS * 32;

__device__ __forceinline__ int ct_slot(int tile, int r)
{
    return tile * CT_TILE + (threadIdx.x >> 5) * CT_WSPAN + r * 32 + (threadIdx.x & 31);
}

// Sum over the block (every thread gets it).
__device__ __forceinline__ int block_sum(int v, int *sh)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(SKID_FULL, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    int t = 0;
    for (int k = 0; k < nw; ++k) t += sh[k];
    return t;
}

// Exclusive prefix of per-warp counts in warp order (every thread gets its
// warp's).
__device__ __forceinline__ int warp_offset(int wc, int *sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = wc;
    __syncthreads();
    int before = 0;
    for (int k = 0; k < w; ++k) before += sh[k];
    return before;
}

// The density floor over touched copies (smooth1.c:460-461).
__global__ void floor_kernel(const float4 *__restrict__ ccoef,
                             const unsigned char *__restrict__ touched, const int *d_n,
                             unsigned *d_floor)
{
    int n = *d_n;
    unsigned best = 0xffffffffu;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (touched[i]) best = min(best, f2ord(ccoef[i].z));
    best = __reduce_min_sync(SKID_FULL, best);
    if ((threadIdx.x & 31) == 0 && best != 0xffffffffu) atomicMin(d_floor, best);
}

// Keep flags (smooth1.c:460-470 with the floor over the touched copies), first-step zeroed densities, touched reset; per-tile kept
// counts.  Block 0 also accumulates the step's algorithmic field bytes.
__global__ void __launch_bounds__(CT_THREADS)
cut_tiles_kernel(float4 *__restrict__ cpos, float4 *__restrict__ ccoef,
                 unsigned char *__restrict__ touched, const int *d_n, const unsigned *d_floor,
                 int initial, int nocut, int *__restrict__ keep, float *__restrict__ final_rho,
                 int *__restrict__ blk, const int *d_nA, double *fbytes)
{
    __shared__ int sh[32];
    const int n = *d_n;
    const unsigned fl = *d_floor;
    const float fScatDens = fl == 0xffffffffu ? 0.0f : ord2f(fl);
    int kept = 0;
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(blockIdx.x, j);
        if (i >= n) break;
        float4 c = ccoef[i];
        bool t = touched[i] != 0;
        if (t) touched[i] = 0;
        int k = 1;
        if (!nocut) {
            if (initial) {
                unsigned bits = __float_as_uint(c.w);
                if (!t && (bits & ORIG_FLAG) && final_rho) final_rho[bits & ~ORIG_FLAG] = 0.0f;
                // a copy that reached no mover counts as density 0 (smooth1.c:463-470)
                float r = t ? c.z : 0.0f;
                k = r >= fScatDens;
            } else {
                k = c.z >= fScatDens;
            }
            // a copy cut now stays in its slot until the next compaction: an
            // empty ball (no mover is inside it) and density -inf (never
            // kept again)
            if (!k && c.z != -INFINITY) {
                cpos[i].w = 0.0f;
                ccoef[i].z = -INFINITY;
            }
        }
        keep[i] = k;
        kept += k;
    }
    kept = block_sum(kept, sh);
    if (threadIdx.x == 0) {
        blk[blockIdx.x] = kept;
        if (blockIdx.x == 0 && fbytes) {
            fbytes[0] += 24.0 * (double)*d_nA + 20.0 * (double)n;
            fbytes[1] += 1.0;
        }
    }
}

// Stable compaction into the spare arrays: tile b starts at the sum of the
// counts of tiles before it.  Block 0 publishes the live count in *d_n2 and
// resets the density floor for the next step.  Nothing is written when
// nothing was cut, or when compaction is deferred (compact = 0, one block:
// the cut copies stay marked in their slots).
__global__ void __launch_bounds__(CT_THREADS)
compact_tiles_kernel(const int *__restrict__ keep, const int *__restrict__ blk, int nb,
                     const int *d_n, int *d_n2, unsigned *d_floor, int compact,
                     const float4 *__restrict__ cpos, const float4 *__restrict__ ccoef,
                     float4 *__restrict__ cpos2, float4 *__restrict__ ccoef2)
{
    __shared__ int sh[32];
    const int n = *d_n;
    const int b = blockIdx.x;
    int pre = 0, all = 0;
    for (int k = threadIdx.x; k < nb; k += CT_THREADS) {
        int v = blk[k];
        all += v;
        if (k < b) pre += v;
    }
    pre = block_sum(pre, sh);
    all = block_sum(all, sh);
    if (b == 0 && threadIdx.x == 0) {
        *d_n2 = all;
        *d_floor = 0xffffffffu;
    }
    if (!compact || all == n) return;
    const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
    unsigned m[CT_ITEMS];
    int wc = 0;
#pragma unroll
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(b, j);
        m[j] = __ballot_sync(SKID_FULL, i < n && keep[i]);
        wc += __popc(m[j]);
    }
    int o = pre + warp_offset(wc, sh);
#pragma unroll
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(b, j);
        if ((m[j] >> (threadIdx.x & 31)) & 1u) {
            const int d = o + __popc(m[j] & lt);
            cpos2[d] = cpos[i];
            ccoef2[d] = ccoef[i];
        }
        o += __popc(m[j]);
    }
}

// Copy the compacted arrays back (a captured graph always reads the primary
// arrays); the last block to finish publishes the count and marks the tree
// dirty, after every block has read the old count.
__global__ void copyback_tiles_kernel(int *d_n, const int *d_n2, float4 *__restrict__ cpos,
                                      float4 *__restrict__ ccoef,
                                      const float4 *__restrict__ cpos2,
                                      const float4 *__restrict__ ccoef2, int *d_dirty, int *d_done)
{
    const int n = *d_n, n2 = *d_n2;
    if (n2 == n) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x) {
        cpos[j] = cpos2[j];
        ccoef[j] = ccoef2[j];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(d_done, 1) == (int)gridDim.x - 1) {
            *d_n = n2;
            *d_dirty = 1;
            *d_done = 0;
        }
    }
}

// kdPruneInactive's test (kd.c:752-762) per active slot, in cut tiles, with
// per-tile survivor counts.
__global__ void __launch_bounds__(CT_THREADS)
prune_flag_kernel(const float4 *__restrict__ mpos, const float4 *__restrict__ mold,
                  const int *__restrict__ act, const int *d_nA, float3 hP, float fCvg2,
                  int *__restrict__ keep, int *__restrict__ blk)
{
    __shared__ int sh[32];
    const int n = *d_nA;
    int kept = 0;
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(blockIdx.x, j);
        if (i >= n) break;
        int m = act[i];
        float4 r = mpos[m], o = mold[m];
        float dx = fsub(r.x, o.x), dy = fsub(r.y, o.y), dz = fsub(r.z, o.z);
        if (dx > hP.x) dx = fsub(dx, fmul(2.0f, hP.x));
        if (dx <= -hP.x) dx = fadd(dx, fmul(2.0f, hP.x));
        if (dy > hP.y) dy = fsub(dy, fmul(2.0f, hP.y));
        if (dy <= -hP.y) dy = fadd(dy, fmul(2.0f, hP.y));
        if (dz > hP.z) dz = fsub(dz, fmul(2.0f, hP.z));
        if (dz <= -hP.z) dz = fadd(dz, fmul(2.0f, hP.z));
        int k = d2of(dx, dy, dz) >= fCvg2;
        keep[i] = k;
        kept += k;
    }
    kept = block_sum(kept, sh);
    if (threadIdx.x == 0) blk[blockIdx.x] = kept;
}

// Survivors get rOld reset (kd.c:785-789) and the Hilbert key of their
// current position at their compacted slot (tile b starts after the
// survivors of the tiles before it; slots [0, survivors) are all written and
// only those are sorted).  Block 0 publishes the survivor count in *d_nA2.
__global__ void __launch_bounds__(CT_THREADS)
prune_scatter_kernel(const int *__restrict__ keep, const int *__restrict__ blk, int nb,
                     const int *d_nA, int *d_nA2, const int *__restrict__ act,
                     const float4 *__restrict__ mpos, float4 *__restrict__ mold, float3 lo,
                     float3 inv, int hil, uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    __shared__ int sh[32];
    const int n = *d_nA;
    const int b = blockIdx.x;
    int pre = 0, all = 0;
    for (int k = threadIdx.x; k < nb; k += CT_THREADS) {
        int v = blk[k];
        all += v;
        if (k < b) pre += v;
    }
    pre = block_sum(pre, sh);
    all = block_sum(all, sh);
    if (b == 0 && threadIdx.x == 0) *d_nA2 = all;
    const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
    unsigned msk[CT_ITEMS];
    int wc = 0;
#pragma unroll
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(b, j);
        msk[j] = __ballot_sync(SKID_FULL, i < n && keep[i]);
        wc += __popc(msk[j]);
    }
    int o = pre + warp_offset(wc, sh);
#pragma unroll
    for (int j = 0; j < CT_ITEMS; ++j) {
        const int i = ct_slot(b, j);
        if ((msk[j] >> (threadIdx.x & 31)) & 1u) {
            const int d = o + __popc(msk[j] & lt);
            int m = act[i];
            float4 p = mpos[m];
            mold[m] = p;
            // the top 32 bits of the Hilbert key (10 to 11 levels) are
            // enough to give each warp a compact set of movers
            keys[d] = curve_top32(make_float3(p.x, p.y, p.z), lo, inv, hil != 0);
            vals[d] = (uint32_t)m;
        }
        o += __popc(msk[j]);
    }
}

// Keys (top 32 bits of the Hilbert or Morton key) of the active movers'
// current positions, in active order.
__global__ void resort_keys_kernel(const int *__restrict__ act, const int *d_nA,
                                   const float4 *__restrict__ mpos, float3 lo, float3 inv, int hil,
                                   uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    const int n = *d_nA;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int m = act[i];
        float4 p = mpos[m];
        keys[i] = curve_top32(make_float3(p.x, p.y, p.z), lo, inv, hil != 0);
        vals[i] = (uint32_t)m;
    }
}

// The sorted movers become the active list; block 0 publishes the count
// (the other blocks read only *d_n2).
__global__ void act_from_sorted(const uint32_t *__restrict__ vals, const int *d_n2,
                                int *__restrict__ act, int *d_n)
{
    int n2 = *d_n2;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x)
        act[j] = (int)vals[j];
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n = n2;
}

float ord_to_float(unsigned u)
{
    unsigned v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &v, 4);
    return f;
}

}  // namespace

cudaError_t build_copies(const float4 *spos, const float *ball2, const float *rho, const int *sidx,
                         int ns, float3 L, float3 boxlo, float3 boxhi, bool periodic,
                         CopyState &C, SortScratch &ss, int *nCopies, cudaStream_t st, bool hil)
{
    cudaError_t e;
    if ((e = dalloc(C.mask, ns)) || (e = dalloc(C.cnt, ns)) || (e = dalloc(C.off, ns)))
        return e;
    copy_count_kernel<<<grid_for(ns), 256, 0, st>>>(spos, ball2, ns, L, boxlo, boxhi, periodic ? 1 : 0, C.mask.p, C.cnt.p); skid::note_launch();
    if ((e = scan_exclusive(C.cnt.p, C.off.p, ns, C.d_n, ss, st))) return e;
    int nc = 0;
    if ((e = cudaMemcpyAsync(&nc, C.d_n, sizeof(int), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    if ((e = C.alloc(nc))) return e;
    copy_write_kernel<<<grid_for(ns), 256, 0, st>>>(spos, ball2, rho, sidx, C.mask.p, C.off.p, ns, L, C.cpos2.p, C.ccoef2.p); skid::note_launch();
    // Hilbert order of the copy positions (replicas lie just outside the box)
    if ((e = dalloc(ss.k0, nc)) || (e = dalloc(ss.k1, nc)) || (e = dalloc(ss.v0, nc)) ||
        (e = dalloc(ss.v1, nc)) || (e = dalloc(ss.box, 8)))
        return e;
    if ((e = bbox_of(C.cpos2.p, nc, ss.box.p, st))) return e;
    unsigned hb[6];
    if ((e = cudaMemcpyAsync(hb, ss.box.p, sizeof(hb), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    float3 lo = make_float3(ord_to_float(hb[0]), ord_to_float(hb[1]), ord_to_float(hb[2]));
    float3 hi = make_float3(ord_to_float(hb[3]), ord_to_float(hb[4]), ord_to_float(hb[5]));
    float ext = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), fmaxf(hi.z - lo.z, 1e-30f));
    float s = 2097151.0f / ext;
    copy_keys_kernel<<<grid_for(nc), 256, 0, st>>>(C.cpos2.p, nc, lo, make_float3(s, s, s), hil ? 1 : 0, ss.k0.p, ss.v0.p); skid::note_launch();
    if ((e = radix_sort(ss, nc, 63, st))) return e;
    copy_permute_kernel<<<grid_for(nc), 256, 0, st>>>(ss.v0.p, nc, C.cpos2.p, C.ccoef2.p, C.cpos.p, C.ccoef.p); skid::note_launch();
    if ((e = cudaMemsetAsync(C.touched.p, 0, C.cap, st))) return e;
    if ((e = cudaMemsetAsync(C.d_dirty, 0, sizeof(int), st))) return e;
    if ((e = cudaMemsetAsync(C.d_floor, 0xff, sizeof(unsigned), st))) return e;
    if ((e = cudaMemcpyAsync(C.d_n2, C.d_n, sizeof(int), cudaMemcpyDeviceToDevice, st))) return e;
    *nCopies = nc;
    return cudaGetLastError();
}

cudaError_t scatter_cut(CopyState &C, bool initial, bool nocut, float *final_rho, const int *d_nA,
                        double *d_fbytes, bool compact, cudaStream_t st)
{
    const int nb = (C.cap + CT_TILE - 1) / CT_TILE;
    if (C.blk.n < (size_t)nb) return cudaErrorInvalidValue;
    floor_kernel<<<grid_for(C.cap), 256, 0, st>>>(C.ccoef.p, C.touched.p, C.d_n, C.d_floor); skid::note_launch();
    cut_tiles_kernel<<<nb, CT_THREADS, 0, st>>>(C.cpos.p, C.ccoef.p, C.touched.p, C.d_n, C.d_floor,
                                                initial ? 1 : 0, nocut ? 1 : 0, C.keep.p, final_rho,
                                                C.blk.p, d_nA, d_fbytes); skid::note_launch();
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    if (nocut) {
        if ((e = cudaMemsetAsync(C.d_floor, 0xff, sizeof(unsigned), st))) return e;
        return cudaMemcpyAsync(C.d_n2, C.d_n, sizeof(int), cudaMemcpyDeviceToDevice, st);
    }
    compact_tiles_kernel<<<compact ? nb : 1, CT_THREADS, 0, st>>>(C.keep.p, C.blk.p, nb, C.d_n, C.d_n2,
                                                                  C.d_floor, compact ? 1 : 0, C.cpos.p,
                                                                  C.ccoef.p, C.cpos2.p, C.ccoef2.p); skid::note_launch();
    if (!compact) return cudaGetLastError();
    copyback_tiles_kernel<<<grid_for(C.cap), 256, 0, st>>>(C.d_n, C.d_n2, C.cpos.p, C.ccoef.p, C.cpos2.p,
                                                           C.ccoef2.p, C.d_dirty, C.d_done); skid::note_launch();
    return cudaGetLastError();
}

// Global re-sort of the active movers between prunes by the Hilbert key of
// their current positions (the same 32-bit key as the prune's; equal keys keep
// their order).  A mover that crosses a high-level curve boundary has to move
// far in the order, which only a global sort does: a tile-local sort, or a
// coarser key, loses most of the gain.
cudaError_t mover_resort(MoverState &m, float3 keylo, float3 keyinv, SortScratch &ss,
                         cudaStream_t st, int bound, bool hil)
{
    cudaError_t e;
    int cap = bound > 0 && bound < m.cap ? bound : m.cap;
    // sort scratch for cap keys: the eager first iteration can re-sort before
    // its prune has sized it (no allocation happens in a captured graph, whose
    // sizes the eager iteration already set)
    if ((e = dalloc(ss.k0, cap)) || (e = dalloc(ss.k1, cap)) || (e = dalloc(ss.v0, cap)) ||
        (e = dalloc(ss.v1, cap)))
        return e;
    resort_keys_kernel<<<grid_for(cap), 256, 0, st>>>(m.act.p, m.d_nA, m.mpos.p, keylo, keyinv,
                                                      hil ? 1 : 0, ss.k0.p, ss.v0.p); skid::note_launch();
    if ((e = radix_sort(ss, cap, 32, st, m.d_nA))) return e;
    act_from_sorted<<<grid_for(cap), 256, 0, st>>>(ss.v0.p, m.d_nA, m.act.p, m.d_nA); skid::note_launch();
    return cudaGetLastError();
}

cudaError_t mover_prune(MoverState &m, float3 period, float3 keylo, float3 keyinv, float fCvg,
                        SortScratch &ss, cudaStream_t st, int bound, bool hil)
{
    cudaError_t e;
    int cap = bound > 0 && bound < m.cap ? bound : m.cap;
    // sort scratch for cap keys (allocated on the first, uncaptured call)
    if ((e = dalloc(ss.k0, cap)) || (e = dalloc(ss.k1, cap)) || (e = dalloc(ss.v0, cap)) ||
        (e = dalloc(ss.v1, cap)))
        return e;
    float3 hP = make_float3((float)(0.5 * (double)period.x), (float)(0.5 * (double)period.y),
                            (float)(0.5 * (double)period.z));
    float fCvg2 = fCvg * fCvg;
    int g = grid_for(cap);
    const int nb = (cap + CT_TILE - 1) / CT_TILE;
    if ((e = dalloc(m.blk, (size_t)nb))) return e;
    prune_flag_kernel<<<nb, CT_THREADS, 0, st>>>(m.mpos.p, m.mold.p, m.act.p, m.d_nA, hP, fCvg2,
                                                 m.keep.p, m.blk.p); skid::note_launch();
    prune_scatter_kernel<<<nb, CT_THREADS, 0, st>>>(m.keep.p, m.blk.p, nb, m.d_nA, m.d_nA2, m.act.p,
                                                    m.mpos.p, m.mold.p, keylo, keyinv, hil ? 1 : 0,
                                                    ss.k0.p, ss.v0.p); skid::note_launch();
    // an even number of digit passes leaves the result in (k0, v0), so a
    // captured graph replays consistently; only the surviving movers' keys
    // (the first *d_nA2 slots) are sorted
    if ((e = radix_sort(ss, cap, 32, st, m.d_nA2))) return e;
    act_from_sorted<<<g, 256, 0, st>>>(ss.v0.p, m.d_nA2, m.act.p, m.d_nA); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
