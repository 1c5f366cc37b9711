// Device tree build: Hilbert- (or Morton-) sorted points bucketed into leaves of one warp
// (32 points) under an implicit complete binary tree (heap numbering of
// kd.h:6-15).  Replaces the reference's median-split kd build
// (kdBuildTree/kdBuildMoveTree, kd.c:225-552): any tree gives the same search
// results; this one is built with one sort and one up-pass.
//
// Node records (float4 pairs):
//   lo/hi   : tight box of the points below; lo.w = max ball2 below
//   blo/bhi : box of the balls below (x -/+ sqrt(ball2)), scatterer trees only
#include <cfloat>

#include "internal.h"

namespace skid {

namespace {

__global__ void bbox_kernel(const float4 *__restrict__ p, int n, unsigned *box)
{
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = p[i];
        mn[0] = fminf(mn[0], q.x); mx[0] = fmaxf(mx[0], q.x);
        mn[1] = fminf(mn[1], q.y); mx[1] = fmaxf(mx[1], q.y);
        mn[2] = fminf(mn[2], q.z); mx[2] = fmaxf(mx[2], q.z);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(SKID_FULL, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(SKID_FULL, mx[d], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int d = 0; d < 3; ++d) {
            atomicMin(&box[d], f2ord(mn[d]));
            atomicMax(&box[3 + d], f2ord(mx[d]));
        }
    }
}

__global__ void curve_kernel(const float4 *__restrict__ p, int n, const unsigned *box, int hil,
                             uint64_t *keys, uint32_t *vals)
{
    float3 lo = make_float3(ord2f(box[0]), ord2f(box[1]), ord2f(box[2]));
    float3 hi = make_float3(ord2f(box[3]), ord2f(box[4]), ord2f(box[5]));
    float ext = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), fmaxf(hi.z - lo.z, 1e-30f));
    float s = 2097151.0f / ext;
    float3 inv = make_float3(s, s, s);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = p[i];
        keys[i] = curve63(make_float3(q.x, q.y, q.z), lo, inv, hil != 0);
        vals[i] = (uint32_t)i;
    }
}

__global__ void gather_sorted(const float4 *__restrict__ p, const uint32_t *__restrict__ perm,
                              int n, float4 *out, uint32_t *perm_out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t j = perm[i];
        out[i] = p[j];
        perm_out[i] = j;
    }
}

// One thread per leaf slot: leaf boxes, then a last-arriver walk up the heap.
// ball2 (sorted order) builds ball boxes when given; aux (sorted order, x =
// ball2, w = live-copy mask bits) is the alternative source for refits.
__global__ void upward_kernel(const float4 *__restrict__ pos, const float *__restrict__ ball2,
                              const float4 *__restrict__ aux, int ballw, int n_host, const int *d_n,
                              int leafBase, float4 *lo, float4 *hi, float4 *blo, float4 *bhi,
                              int *flag, int *d_dirty)
{
    int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= leafBase) return;
    if (d_dirty && !*d_dirty) return;
    int n = d_n ? *d_n : n_host;
    float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX);
    float4 h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
    float4 bl = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
    float4 bh = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
    // max ball2 (lo.w) needs ball data; ball boxes also need allocated arrays
    bool hasb = (ball2 != nullptr) || (aux != nullptr) || ballw;
    bool balls = hasb && blo != nullptr && bhi != nullptr;
    int b = leaf * SKID_LEAF, e = min(b + SKID_LEAF, n);
    for (int i = b; i < e; ++i) {
        float4 q = pos[i];
        float b2 = 0.0f;
        bool live = true;
        if (ballw) {
            b2 = q.w;
        } else if (aux) {
            float4 a = aux[i];
            b2 = a.x;
            live = __float_as_uint(a.w) != 0u;
        } else if (ball2) {
            b2 = ball2[i];
        }
        if (!live) continue;
        l.x = fminf(l.x, q.x); l.y = fminf(l.y, q.y); l.z = fminf(l.z, q.z);
        h.x = fmaxf(h.x, q.x); h.y = fmaxf(h.y, q.y); h.z = fmaxf(h.z, q.z);
        if (hasb) l.w = fmaxf(l.w, b2);
        if (balls) {
            // ball radius rounded up so the box contains every d2 < b2 point
            float r = sqrtf(b2) * (1.0f + 1e-6f) + 1e-30f;
            r += 4.8e-7f * (fabsf(q.x) + fabsf(q.y) + fabsf(q.z) + r);
            bl.x = fminf(bl.x, q.x - r); bl.y = fminf(bl.y, q.y - r); bl.z = fminf(bl.z, q.z - r);
            bh.x = fmaxf(bh.x, q.x + r); bh.y = fmaxf(bh.y, q.y + r); bh.z = fmaxf(bh.z, q.z + r);
        }
    }
    int node = leafBase + leaf;
    lo[node] = l;
    hi[node] = h;
    if (balls) { blo[node] = bl; bhi[node] = bh; }
    __threadfence();
    if (leafBase == 1 && d_dirty) *d_dirty = 0;   // the only leaf is the root
    node >>= 1;
    while (node >= 1) {
        int old = atomicAdd(&flag[node], 1);
        if (old == 0) return;
        // the second arrival finishes the node and clears its flag for the
        // next refit (each node has exactly two arrivals per launch)
        flag[node] = 0;
        __threadfence();
        float4 l0 = __ldcg(&lo[2 * node]), l1 = __ldcg(&lo[2 * node + 1]);
        float4 h0 = __ldcg(&hi[2 * node]), h1 = __ldcg(&hi[2 * node + 1]);
        lo[node] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z),
                               fmaxf(l0.w, l1.w));
        hi[node] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
        if (balls) {
            float4 a0 = __ldcg(&blo[2 * node]), a1 = __ldcg(&blo[2 * node + 1]);
            float4 c0 = __ldcg(&bhi[2 * node]), c1 = __ldcg(&bhi[2 * node + 1]);
            blo[node] = make_float4(fminf(a0.x, a1.x), fminf(a0.y, a1.y), fminf(a0.z, a1.z), 0.0f);
            bhi[node] = make_float4(fmaxf(c0.x, c1.x), fmaxf(c0.y, c1.y), fmaxf(c0.z, c1.z), 0.0f);
        }
        __threadfence();
        // the root is finished after every leaf thread has read d_dirty
        if (node == 1 && d_dirty) *d_dirty = 0;
        node >>= 1;
    }
}

}  // namespace

cudaError_t bbox_of(const float4 *pts, int n, unsigned *d_box6, cudaStream_t st)
{
    // order-preserving bit patterns: the three minima start at all ones, the
    // three maxima at zero (set on the device, no host memory involved)
    cudaError_t e = cudaMemsetAsync(d_box6, 0xff, 3 * sizeof(unsigned), st);
    if (!e) e = cudaMemsetAsync(d_box6 + 3, 0, 3 * sizeof(unsigned), st);
    if (e) return e;
    int blocks = min((n + 255) / 256, num_sms() * 4);
    if (blocks < 1) blocks = 1;
    bbox_kernel<<<blocks, 256, 0, st>>>(pts, n, d_box6); skid::note_launch();
    return cudaGetLastError();
}

static int leaf_base_for(int n)
{
    int nLeaf = (n + SKID_LEAF - 1) / SKID_LEAF;
    int p = 1;
    while (p < nLeaf) p <<= 1;
    return p;
}

cudaError_t tree_build(Tree &t, const float4 *pts, int n, bool balls, SortScratch &s,
                       cudaStream_t st, bool hil)
{
    cudaError_t e;
    t.n = n;
    t.nLeaf = (n + SKID_LEAF - 1) / SKID_LEAF;
    t.leafBase = leaf_base_for(n);
    size_t nodes = 2 * (size_t)t.leafBase;
    if ((e = dalloc(t.pos, n)) || (e = dalloc(t.perm, n)) || (e = dalloc(t.lo, nodes)) ||
        (e = dalloc(t.hi, nodes)) || (e = dalloc(t.flag, nodes)))
        return e;
    t.flag_clear = false;
    if (balls) {
        if ((e = dalloc(t.blo, nodes)) || (e = dalloc(t.bhi, nodes))) return e;
    }
    if (n > 0) {
        int blocks = min((n + 255) / 256, num_sms() * 8);
        if ((e = curve_order(pts, n, s, st, hil))) return e;
        gather_sorted<<<blocks, 256, 0, st>>>(pts, s.v0.p, n, t.pos.p, t.perm.p); skid::note_launch();
    }
    return tree_refit(t, nullptr, nullptr, nullptr, st);
}

cudaError_t curve_order(const float4 *pts, int n, SortScratch &s, cudaStream_t st, bool hil)
{
    cudaError_t e;
    if (n <= 0) return cudaSuccess;
    if ((e = dalloc(s.k0, n)) || (e = dalloc(s.k1, n)) || (e = dalloc(s.v0, n)) ||
        (e = dalloc(s.v1, n)) || (e = dalloc(s.box, 8)))
        return e;
    unsigned *dbox = s.box.p;
    if ((e = bbox_of(pts, n, dbox, st))) return e;
    int blocks = min((n + 255) / 256, num_sms() * 8);
    curve_kernel<<<blocks, 256, 0, st>>>(pts, n, dbox, hil ? 1 : 0, s.k0.p, s.v0.p); skid::note_launch();
    return radix_sort(s, n, 63, st);
}

cudaError_t tree_refit(Tree &t, const float4 *pos, const float4 *aux, const int *d_n,
                       cudaStream_t st, bool ballw, int *d_dirty)
{
    cudaError_t e = cudaSuccess;
    // arrival flags start zero (allocation) and every launch leaves them zero
    if (!t.flag_clear) {
        if ((e = cudaMemsetAsync(t.flag.p, 0, 2 * (size_t)t.leafBase * sizeof(int), st))) return e;
        t.flag_clear = true;
    }
    int threads = 128;
    int blocks = (t.leafBase + threads - 1) / threads;
    bool nb = t.blo.n < 2 * (size_t)t.leafBase || t.bhi.n < 2 * (size_t)t.leafBase;
    upward_kernel<<<blocks, threads, 0, st>>>(pos ? pos : t.pos.p, nullptr, aux, ballw ? 1 : 0,
                                              t.n, d_n, t.leafBase, t.lo.p, t.hi.p,
                                              nb ? nullptr : t.blo.p, nb ? nullptr : t.bhi.p,
                                              t.flag.p, d_dirty); skid::note_launch();
    return cudaGetLastError();
}

cudaError_t tree_shape(Tree &t, int n, bool balls)
{
    cudaError_t e;
    t.n = n;
    t.nLeaf = (n + SKID_LEAF - 1) / SKID_LEAF;
    t.leafBase = leaf_base_for(n);
    size_t nodes = 2 * (size_t)t.leafBase;
    if ((e = dalloc(t.lo, nodes)) || (e = dalloc(t.hi, nodes)) || (e = dalloc(t.flag, nodes)))
        return e;
    t.flag_clear = false;
    if (balls && ((e = dalloc(t.blo, nodes)) || (e = dalloc(t.bhi, nodes)))) return e;
    return cudaSuccess;
}

}  // namespace skid
