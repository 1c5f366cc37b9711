// k-nearest-neighbour ball radii (fBall2) of every point of a tree, among the
// tree's own points, self included (smDensityInit/smBallSearch,
// smooth1.c:41-243).  Only the k-th smallest squared distance is kept: the
// density gather needs fBall2 alone, and that value does not depend on how
// equal distances are ordered.
//
// One warp per leaf of 32 query points, one query per lane.  Each lane keeps
// a max-heap of its k best squared distances in shared memory (slot i of
// lane l at i*32+l, so every heap access is bank-conflict free).  The warp
// first scans its own leaf, then climbs to the root visiting each sibling
// subtree depth-first (the search order of smBallSearch, smooth1.c:89-127),
// entering a node when any lane's heap bound reaches its box.  The last five
// levels of a subtree are tested one leaf per lane against the query leaf's
// box and the warp's largest bound; at a leaf only candidates within that
// bound of the query box are compacted and tested.
#include <cfloat>

#include <mutex>

#include "internal.h"

namespace skid {

namespace {

constexpr int KNN_WARPS = 4;

struct KnnLane {
    float3 q;       // query
    float thr;      // current k-th smallest (heap top)
    float *heap;    // this lane's heap base (stride 32)
};

__device__ __forceinline__ void heap_replace_top(float *heap, int k, float d)
{
    int i = 0;
    for (;;) {
        int c = 2 * i + 1;
        if (c >= k) break;
        float vc = heap[c * 32];
        if (c + 1 < k) {
            float vr = heap[(c + 1) * 32];
            if (vr > vc) { vc = vr; ++c; }
        }
        if (vc <= d) break;
        heap[i * 32] = vc;
        i = c;
    }
    heap[i * 32] = d;
}

// Process one leaf: candidates staged in shared memory, every lane tests all
// of them.  With a query box (filter), lane j first drops candidate j when
// its distance to the box is at least the warp's largest heap bound tmax:
// no lane can take it; the survivors are compacted in order.
__device__ __forceinline__ void knn_leaf(const TreeView &t, int node, float4 blo, float4 bhi,
                                         KnnLane &ln, int k, float3 L, float3 hL, bool per,
                                         float4 *cand, int lane, bool filter, float4 qlo,
                                         float4 qhi, float tmax)
{
    int leaf = node - t.leafBase;
    if (leaf >= t.nLeaf) return;
    int base = leaf * SKID_LEAF;
    int cnt = min(SKID_LEAF, t.n - base);
    float4 c4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool rel = lane < cnt;
    if (rel) {
        c4 = t.pos[base + lane];
        if (filter) rel = box_lb(make_float3(c4.x, c4.y, c4.z), qlo, qhi, L, per) < tmax;
    }
    const unsigned R = __ballot_sync(SKID_FULL, rel);
    cnt = __popc(R);
    __syncwarp();
    if (rel) cand[__popc(R & ((1u << lane) - 1u))] = c4;
    __syncwarp();
    int cx = img_class(ln.q.x, blo.x, bhi.x, hL.x);
    int cy = img_class(ln.q.y, blo.y, bhi.y, hL.y);
    int cz = img_class(ln.q.z, blo.z, bhi.z, hL.z);
    bool mixed = (cx == 2) | (cy == 2) | (cz == 2);
    if (__any_sync(SKID_FULL, mixed)) {
        for (int j = 0; j < cnt; ++j) {
            float4 c = cand[j];
            float dx = img_dx(ln.q.x, c.x, L.x, hL.x);
            float dy = img_dx(ln.q.y, c.y, L.y, hL.y);
            float dz = img_dx(ln.q.z, c.z, L.z, hL.z);
            float d2 = d2of(dx, dy, dz);
            if (d2 < ln.thr) {
                heap_replace_top(ln.heap, k, d2);
                ln.thr = ln.heap[0];
            }
        }
        return;
    }
    float sx = cx == 0 ? ln.q.x : (cx < 0 ? fsub(ln.q.x, L.x) : fadd(ln.q.x, L.x));
    float sy = cy == 0 ? ln.q.y : (cy < 0 ? fsub(ln.q.y, L.y) : fadd(ln.q.y, L.y));
    float sz = cz == 0 ? ln.q.z : (cz < 0 ? fsub(ln.q.z, L.z) : fadd(ln.q.z, L.z));
#pragma unroll 4
    for (int j = 0; j < cnt; ++j) {
        float4 c = cand[j];
        float d2 = d2of(fsub(sx, c.x), fsub(sy, c.y), fsub(sz, c.z));
        if (d2 < ln.thr) {
            heap_replace_top(ln.heap, k, d2);
            ln.thr = ln.heap[0];
        }
    }
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(SKID_FULL, v, o));
    return v;
}

// Heaps live in shared memory after the candidate buffers, or -- for k too
// large for one warp's heaps to fit -- in global scratch (gheap, one slab per
// resident warp).
__global__ void __launch_bounds__(KNN_WARPS * 32, 6)
knn_kernel(TreeView t, int k, float3 L, float3 hL, bool per, int logLeafBase, int subShift,
           float *__restrict__ ball2, int *work, float *gheap)
{
    extern __shared__ float4 smem4[];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int nw = blockDim.x >> 5;
    float4 *cand = smem4 + w * SKID_LEAF;
    float *heaps = gheap ? gheap + (size_t)blockIdx.x * nw * k * 32
                         : reinterpret_cast<float *>(smem4 + nw * SKID_LEAF);
    const int rootLo = t.leafBase >> subShift;
    KnnLane ln;
    ln.heap = heaps + (size_t)w * k * 32 + lane;
    for (;;) {
        int leaf = 0;
        if (lane == 0) leaf = atomicAdd(work, 1);
        leaf = __shfl_sync(SKID_FULL, leaf, 0);
        if (leaf >= t.nLeaf) break;
        int base = leaf * SKID_LEAF;
        int qi = base + lane;
        bool valid = qi < t.n;
        float4 qp = t.pos[valid ? qi : base];
        ln.q = make_float3(qp.x, qp.y, qp.z);
        for (int i = 0; i < k; ++i) ln.heap[i * 32] = FLT_MAX;
        ln.thr = FLT_MAX;
        int own = t.leafBase + leaf;
        const float4 qlo = t.lo[own], qhi = t.hi[own];   // the queries' box
        knn_leaf(t, own, qlo, qhi, ln, k, L, hL, per, cand, lane, false, qlo, qhi, FLT_MAX);
        int cell = own;
        while (cell > 1) {
            int cp = cell ^ 1;
            int end = next_node(cp);
            for (;;) {
                if (cp >= rootLo) {
                    // a subtree of at most 2^subShift leaves: one lane per
                    // leaf against the queries' box and the largest bound,
                    // then each passing leaf in order with the exact bounds
                    const int sh = logLeafBase - (31 - __clz(cp));
                    const int first = cp << sh;
                    float tmax = warp_max(ln.thr);
                    bool pass = false;
                    if (lane < (1 << sh) && first + lane - t.leafBase < t.nLeaf)
                        pass = boxbox_lb(qlo, qhi, t.lo[first + lane], t.hi[first + lane], L, per) < tmax;
                    for (unsigned lm = __ballot_sync(SKID_FULL, pass); lm; lm &= lm - 1) {
                        const int node = first + __ffs(lm) - 1;
                        float4 blo = t.lo[node], bhi = t.hi[node];
                        bool want = box_lb(ln.q, blo, bhi, L, per) < ln.thr;
                        if (!__any_sync(SKID_FULL, want)) continue;
                        knn_leaf(t, node, blo, bhi, ln, k, L, hL, per, cand, lane, true, qlo, qhi,
                                 warp_max(ln.thr));
                    }
                } else {
                    float4 blo = t.lo[cp], bhi = t.hi[cp];
                    bool want = box_lb(ln.q, blo, bhi, L, per) < ln.thr;
                    if (__any_sync(SKID_FULL, want)) { cp <<= 1; continue; }
                }
                cp = next_node(cp);
                if (cp == end) break;
            }
            cell >>= 1;
        }
        if (valid) ball2[qi] = ln.thr;
    }
}

}  // namespace

cudaError_t knn_ball2(const Tree &t, int k, float3 L, bool per, float *ball2_sorted, int *d_work,
                      DBuf<float> &gheap, cudaStream_t st)
{
    if (t.n <= 0) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    size_t heapBytes = (size_t)k * 32 * sizeof(float);
    size_t candBytes = SKID_LEAF * sizeof(float4);
    int nw = KNN_WARPS;
    while (nw > 1 && (size_t)nw * (candBytes + heapBytes) > (size_t)optin) nw >>= 1;
    bool global = (size_t)nw * (candBytes + heapBytes) > (size_t)optin;
    size_t smem = (size_t)nw * candBytes + (global ? 0 : (size_t)nw * heapBytes);
    // The attribute belongs to the device and is only an upper bound: raise it
    // to the opt-in maximum once per device (contexts on other threads launch
    // with other k).
    static std::mutex attr_mu;
    static bool attr_done[SKID_MAX_DEVICES] = {};
    if (dev < 0 || dev >= SKID_MAX_DEVICES) return cudaErrorInvalidDevice;
    cudaError_t e = cudaSuccess;
    {
        std::lock_guard<std::mutex> lk(attr_mu);
        if (!attr_done[dev]) {
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, knn_kernel);
            if (!e)
                e = cudaFuncSetAttribute(knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         optin - (int)fa.sharedSizeBytes);
            if (!e) attr_done[dev] = true;
        }
    }
    if (e) return e;
    int perSM = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, knn_kernel, nw * 32, smem);
    if (e) return e;
    if (perSM < 1) return cudaErrorInvalidConfiguration;
    int blocks = num_sms() * perSM;
    int need = (t.nLeaf + nw - 1) / nw;
    if (blocks > need) blocks = need;
    float *gh = nullptr;
    if (global) {
        if ((e = dalloc(gheap, (size_t)blocks * nw * k * 32))) return e;
        gh = gheap.p;
    }
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    if ((e = cudaMemsetAsync(d_work, 0, sizeof(int), st))) return e;
    int logLeafBase = 0;
    while ((2 << logLeafBase) <= t.leafBase) ++logLeafBase;
    int subShift = logLeafBase < 5 ? logLeafBase : 5;
    knn_kernel<<<blocks, nw * 32, smem, st>>>(t.view(), k, L, hL, per, logLeafBase, subShift,
                                              ball2_sorted, d_work, gh); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
