// Internal host-side interfaces of libskidgpu: the context and the kernel
// launchers each .cu file provides.  Not part of the public C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace skid {

// Device buffer that remembers its size.
template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
};

template <typename T>
cudaError_t dalloc(DBuf<T> &b, size_t n)
{
    if (b.n >= n && b.p) return cudaSuccess;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = cudaMalloc((void **)&b.p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) b.n = n;
    return e;
}

template <typename T>
void dfree(DBuf<T> &b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

// Scratch for sorting and scans, sized for the largest point set.
struct SortScratch {
    DBuf<uint64_t> k0, k1;
    DBuf<uint32_t> v0, v1;
    DBuf<uint32_t> hist;   // per-block digit counts
    DBuf<int> blk;         // per-block sums for scans
    DBuf<unsigned> box;    // bounding box (ordered uints)
};

// A tree over a point set (kNN, gather, FoF, scoop).
struct Tree {
    int n = 0, nLeaf = 0, leafBase = 1;
    DBuf<float4> pos;      // sorted points
    DBuf<uint32_t> perm;   // sorted slot -> input index
    DBuf<float4> lo, hi;   // point boxes per node
    DBuf<float4> blo, bhi; // ball boxes per node (scatterer trees)
    DBuf<int> flag;        // up-pass arrival counters
    TreeView view() const
    {
        TreeView v;
        v.n = n; v.nLeaf = nLeaf; v.leafBase = leafBase;
        v.pos = pos.p; v.lo = lo.p; v.hi = hi.p;
        return v;
    }
};

// ---- sort.cu ----
// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
// Result lands in (k0, v0) of the scratch.
cudaError_t radix_sort(SortScratch &s, int n, int bits, cudaStream_t st);
// Exclusive scan of int flags/counts; out may alias in; total -> *d_total.
cudaError_t scan_exclusive(const int *in, int *out, int n, int *d_total, SortScratch &s,
                           cudaStream_t st);
int num_sms();

// ---- tree.cu ----
// Build a tree over n points (float4, w carried along).  perm maps sorted
// slots to input indices.  `balls` reserves ball boxes, filled by a refit
// that is given per-slot ball data.
cudaError_t tree_build(Tree &t, const float4 *pts, int n, bool balls, SortScratch &s,
                       cudaStream_t st);
// Recompute leaf and node boxes from pos (t.pos when null) and, when aux is
// given, per-slot ball data (aux.x = ball2, aux.w = live-copy mask; slots
// with an empty mask are left out).  d_n (device) overrides t.n.
cudaError_t tree_refit(Tree &t, const float4 *pos, const float4 *aux, const int *d_n,
                       cudaStream_t st);
// Morton order of n points: sorted permutation lands in s.v0.
cudaError_t morton_order(const float4 *pts, int n, SortScratch &s, cudaStream_t st);
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

// Scatterers in tree (Morton) order, compacted as ScatterCut removes them.
// aux = (fBall2, ih2, fNorm*m, live-copy mask bits).
struct ScatState {
    DBuf<float4> spos, saux, spos2, saux2;
    DBuf<float> srho, srho2;
    DBuf<int> sidx, sidx2;          // iOrder of each slot
    DBuf<unsigned char> touched;    // reached an active mover (non-first passes)
    DBuf<unsigned> tbits;           // copies that reached a mover (first pass)
    DBuf<int> keep, kpos;
    int *d_nS = nullptr;            // live scatterers (device)
    int *d_nS2 = nullptr;
    unsigned *d_floor = nullptr;    // ordered-uint min density (fScatDens)
    int *d_live = nullptr;          // live copies after the cut
};

// Movers: positions by mover index; `act` lists the active ones.
struct MoverState {
    DBuf<float4> mpos, mold;
    DBuf<int> mio;                  // iOrder of each mover
    DBuf<int> act, act2, keep, kpos;
    int *d_nA = nullptr;
    int *d_nA2 = nullptr;
};

struct FieldArgs {
    // scatterers (tree-sorted, compacted): pos (x,y,z,m), aux (b, ih2, fnorm*m, mask)
    const float4 *spos;
    const float4 *saux;
    const float4 *blo, *bhi;     // ball boxes
    const float4 *lo, *hi;       // point boxes (periodic image class at leaves)
    int leafBase;
    const int *d_nS;             // live scatterers
    // movers
    float4 *mpos;                // positions (w unused)
    const int *act;              // active mover indices
    const int *d_nA;
    float3 L, hL;
    bool per;
    float fStep;                 // 0: no move (field probe)
    float3 wrapHi, wrapLo;       // float thresholds of kdMoveParticles' wrap
    float3 period;
    float *acc_out;              // optional [3*nA] field output (probe)
    unsigned char *touched;      // per scatterer slot (non-initial passes)
    unsigned *touched_bits;      // per scatterer slot image bits (initial pass)
    int *d_work;
    unsigned *d_status;
};
cudaError_t field_move(const FieldArgs &a, int max_movers, cudaStream_t st);

// ---- scatter.cu ----
cudaError_t scatter_aux(const float4 *spos, const float *ball2_sorted, int n, float3 L,
                        float3 boxlo, float3 boxhi, bool periodic, float4 *aux, int *d_extra,
                        cudaStream_t st);
// After a move pass: density floor, cut, stable compaction, counts.
cudaError_t scatter_cut(ScatState &s, bool initial, bool nocut, float *final_rho, SortScratch &ss,
                        cudaStream_t st);
cudaError_t mover_prune(MoverState &m, float3 period, float fCvg, SortScratch &ss, cudaStream_t st);

}  // namespace skid
