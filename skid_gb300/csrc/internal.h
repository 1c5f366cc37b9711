// Internal host-side interfaces of libskidgpu: the context and the kernel
// launchers each .cu file provides.  Not part of the public C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"

namespace skid {

// Per-device tables (SM counts, kernel attributes, static scratch addresses)
// are indexed by the CUDA device ordinal below this bound.
constexpr int SKID_MAX_DEVICES = 64;

// Device buffer that remembers its size.
// Device allocation, freeing and graph capture take this process-wide lock:
// cudaMalloc/cudaFree may synchronise the device, which must not happen while
// another host thread's stream is being captured into a graph (batched runs
// drive several contexts from several threads).  Recursive: a capture may
// reach a dalloc that finds its buffer already large enough.
std::recursive_mutex &device_mutex();

// Counts every device (re)allocation made through dalloc, process-wide: a
// captured graph whose count is unchanged still points at live buffers.
unsigned long long alloc_epoch();
void bump_alloc_epoch();

template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
};

template <typename T>
cudaError_t dalloc(DBuf<T> &b, size_t n)
{
    if (b.n >= n && b.p) return cudaSuccess;
    std::lock_guard<std::recursive_mutex> lk(device_mutex());
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    bump_alloc_epoch();
    cudaError_t e = cudaMalloc((void **)&b.p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) b.n = n;
    return e;
}

template <typename T>
void dfree(DBuf<T> &b)
{
    if (!b.p) return;
    std::lock_guard<std::recursive_mutex> lk(device_mutex());
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

// Words of SortScratch::glob: eight passes' digit offsets and tile counters.
constexpr size_t SORT_GLOB_WORDS = 8 * 256 + 8;

// Scratch for sorting and scans, sized for the largest point set.
struct SortScratch {
    DBuf<uint64_t> k0, k1;
    DBuf<uint32_t> v0, v1;
    DBuf<uint32_t> hist;   // per-tile look-back status of a sort pass (256 per tile)
    DBuf<uint32_t> glob;   // SORT_GLOB_WORDS: digit offsets of every pass, tile counters
    DBuf<int> blk;         // per-block sums for scans
    DBuf<unsigned> box;    // bounding box (ordered uints)
    unsigned *d_err = nullptr;   // status word a timed-out wait sets (may be null)
};

// A tree over a point set (kNN, gather, FoF, scoop).
struct Tree {
    int n = 0, nLeaf = 0, leafBase = 1;
    DBuf<float4> pos;      // sorted points
    DBuf<uint32_t> perm;   // sorted slot -> input index
    DBuf<float4> lo, hi;   // point boxes per node
    DBuf<float4> blo, bhi; // ball boxes per node (scatterer trees)
    DBuf<int> flag;        // up-pass arrival counters
    bool flag_clear = false;   // flag holds zeros (each refit leaves it so)
    TreeView view() const
    {
        TreeView v;
        v.n = n; v.nLeaf = nLeaf; v.leafBase = leafBase;
        v.pos = pos.p; v.lo = lo.p; v.hi = hi.p;
        return v;
    }
};

// ---- launch accounting (sort.cu) ----
// Every kernel launch calls note_launch(); launches enqueued while a stream is
// being captured into a graph are not counted (the graph's replays are).
void note_launch(int n = 1);
long long launches_total();
void set_capturing(bool on);

// ---- sort.cu ----
// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
// Result lands in (k0, v0) of the scratch.
// With d_n, only the first min(n, *d_n) keys are sorted (the count is read
// on the device, so a captured graph follows it); the rest are left as they are.
cudaError_t radix_sort(SortScratch &s, int n, int bits, cudaStream_t st, const int *d_n = nullptr);
// Exclusive scan of int flags/counts; out may alias in; total -> *d_total.
cudaError_t scan_exclusive(const int *in, int *out, int n, int *d_total, SortScratch &s,
                           cudaStream_t st);
int num_sms();

// ---- tree.cu ----
// Build a tree over n points (float4, w carried along).  perm maps sorted
// slots to input indices.  `balls` reserves ball boxes, filled by a refit
// that is given per-slot ball data.  Points are ordered by their Hilbert
// key (hil) or Morton key; any order gives the same search results.
cudaError_t tree_build(Tree &t, const float4 *pts, int n, bool balls, SortScratch &s,
                       cudaStream_t st, bool hil = true);
// Recompute leaf and node boxes from pos (t.pos when null).  With aux, ball
// data per slot (aux.x = ball2) also builds the ball boxes and max ball2;
// with ballw the ball2 is pos.w instead.  d_n (device) overrides t.n; with
// d_dirty the refit runs only when *d_dirty is set, and clears it.
cudaError_t tree_refit(Tree &t, const float4 *pos, const float4 *aux, const int *d_n,
                       cudaStream_t st, bool ballw = false, int *d_dirty = nullptr);
// Node arrays for n already-ordered points (no sort).
cudaError_t tree_shape(Tree &t, int n, bool balls);
// Hilbert (hil) or Morton order of n points: sorted permutation lands in s.v0.
cudaError_t curve_order(const float4 *pts, int n, SortScratch &s, cudaStream_t st, bool hil = true);
cudaError_t bbox_of(const float4 *pts, int n, unsigned *d_box6, cudaStream_t st);

// ---- knn.cu ----
// fBall2 of every point of the tree among the tree's points (sorted order).
// Per-lane heaps go to shared memory, or to gheap when k is too large.
cudaError_t knn_ball2(const Tree &t, int k, float3 L, bool per, float *ball2_sorted,
                      int *d_work, DBuf<float> &gheap, cudaStream_t st);

// ---- gather.cu ----
// Symmetric SPH density of every scatterer (sorted order), FP32 Kahan.
cudaError_t density_gather(const Tree &t, const float *ball2_sorted, float3 L, bool per,
                           float *rho_sorted, int *d_work, cudaStream_t st);

// Scatterer copies of the move phase (originals and periodic replicas), in
// Hilbert order of the copy positions, compacted as ScatterCut removes them.
//   cpos  = (x_c, y_c, z_c, fBall2)
//   ccoef = (ih2, fNorm*m, rho, iOrder | 0x80000000 for the original)
struct CopyState {
    int cap = 0;
    DBuf<float4> cpos, ccoef, cpos2, ccoef2;
    DBuf<unsigned char> touched;    // reached an active mover this step
    DBuf<int> keep, kpos;
    DBuf<int> blk;                  // kept copies per cut tile
    DBuf<unsigned> mask;            // build-time image masks
    DBuf<int> cnt, off;             // build-time copy counts / offsets
    int *d_n = nullptr;             // live copies (device)
    int *d_n2 = nullptr;            // live copies after the last cut
    unsigned *d_floor = nullptr;    // ordered-uint min density (fScatDens)
    int *d_dirty = nullptr;         // copies changed since the last refit
    int *d_done = nullptr;          // finished write-back blocks (zero between steps)
    cudaError_t alloc(int n)
    {
        cudaError_t e;
        size_t m = n > 0 ? n : 1;
        if ((e = dalloc(cpos, m)) || (e = dalloc(ccoef, m)) || (e = dalloc(cpos2, m)) ||
            (e = dalloc(ccoef2, m)) || (e = dalloc(touched, m)) || (e = dalloc(keep, m)) ||
            (e = dalloc(kpos, m)) || (e = dalloc(blk, (m + 4095) / 4096)))
            return e;
        cap = (int)m;
        return cudaSuccess;
    }
};

// Movers: positions by mover index; `act` lists the active ones, sorted by
// the Hilbert key of their current positions after every prune.
struct MoverState {
    int cap = 0;
    DBuf<float4> mpos, mold;
    DBuf<int> mio;                  // iOrder of each mover
    DBuf<int> act, act2, keep, kpos;
    DBuf<int> blk;                  // surviving movers per prune tile
    int *d_nA = nullptr;
    int *d_nA2 = nullptr;
};

// Capacity of the split-mover buffers: one-mover-per-warp steps split each
// mover's walk over S warps while (active movers x S) fits in it.
constexpr int FIELD_SPLIT_CAP = 16384;

struct FieldArgs {
    const float4 *cpos, *ccoef;      // copies
    const float4 *blo, *bhi;         // ball boxes of the copy tree
    int leafBase;
    int logLeafBase;                 // depth of the leaves (leafBase = 2^logLeafBase)
    const int *d_nC;                 // live copies
    float4 *mpos;                    // mover positions (w unused)
    const int *act;                  // active mover indices
    const int *d_nA;
    float fStep;                     // 0: no move (field probe)
    float3 wrapHi, wrapLo;           // float thresholds of kdMoveParticles' wrap
    float3 period;
    float *acc_out;                  // optional [3*nA] field output (probe)
    unsigned char *touched;          // per copy slot
    int *d_work;
    unsigned *d_status;
    unsigned long long *stats;       // optional: nodes, leaves, candidate tests, hits
    float *part_acc;                 // split movers' partial fields [FIELD_SPLIT_CAP x 3] (or null)
    int *part_cnt;                   // parts finished per mover [FIELD_SPLIT_CAP], zero between steps
    int G;                           // movers per warp: 32, 16, 8, 4 or 1
};
cudaError_t field_move(const FieldArgs &a, int max_movers, cudaStream_t st);
// The move step alone, from a field computed with fStep = 0 into acc.
cudaError_t move_movers(const FieldArgs &a, const float *acc, float fStep, int max_movers,
                        cudaStream_t st);

// ---- scatter.cu ----
// Copies of the ns scatterers (sorted order) with their densities; sets
// *nCopies and fills C, sorted by Hilbert (hil) or Morton key.
cudaError_t build_copies(const float4 *spos, const float *ball2, const float *rho, const int *sidx,
                         int ns, float3 L, float3 boxlo, float3 boxhi, bool periodic,
                         CopyState &C, SortScratch &ss, int *nCopies, cudaStream_t st,
                         bool hil = true);
// After a move pass: density floor, cut, stable compaction, counts.
// compact = false defers the compaction: cut copies stay marked in their
// slots (empty ball, density -inf) and only the live count is published.
cudaError_t scatter_cut(CopyState &C, bool initial, bool nocut, float *final_rho, const int *d_nA,
                        double *d_fbytes, bool compact, cudaStream_t st);
// Re-sort the active movers by the Hilbert (hil) or Morton key of their
// current positions.
cudaError_t mover_resort(MoverState &m, float3 keylo, float3 keyinv, SortScratch &ss,
                         cudaStream_t st, int bound, bool hil = true);
// Prune converged movers, then re-sort the active ones by key as above.
// bound: active movers at most (the sort and tiles are sized for it).
cudaError_t mover_prune(MoverState &m, float3 period, float3 keylo, float3 keyinv, float fCvg,
                        SortScratch &ss, cudaStream_t st, int bound = -1, bool hil = true);

inline int grid_for(int n, int threads = 256)
{
    int b = (n + threads - 1) / threads;
    int cap = num_sms() * 8;
    if (b > cap) b = cap;
    return b < 1 ? 1 : b;
}

}  // namespace skid
