// Friends-of-friends (kdFoF, kd.c:802-917) as a lock-free union-find.
//
// Edge rule: particles i and j are friends when d2(i->j) < tau^2 or
// d2(j->i) < tau^2 (float, no FMA, periodic image of the query; the
// reference tests the dequeued particle's frame, kd.c:869-876).  Groups are
// the connected components, numbered by ascending smallest member iOrder.
//
// The reference floods breadth-first and takes whole "contained" cells at
// once (INTERCONT, kd.h:217-335, kd.c:888-897), which matters because the
// moved particles of a group sit inside a ball of radius ~fCvg.  Here a node
// whose box diagonal is below tau is a clique; a pre-pass links each clique
// to its children's first points, and a query skips a clique subtree as soon
// as it is already in that clique's component.  Each pair is linked from its
// lower slot, so a query skips every subtree below its own leaf.
#include <cfloat>

#include "ctx.h"

namespace skid {

namespace {

constexpr int F_WARPS = 4;
constexpr int UF_SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ int uf_find(int *par, int x)
{
    for (int it = 0; it < UF_SPIN_LIMIT; ++it) {
        int p = __ldcg(&par[x]);
        if (p == x) return x;
        int gp = __ldcg(&par[p]);
        if (gp != p) par[x] = gp;   // path halving; gp is an ancestor of x
        x = gp;
    }
    return x;
}

__device__ __forceinline__ void uf_union(int *par, int a, int b, unsigned *status)
{
    for (int it = 0; it < UF_SPIN_LIMIT; ++it) {
        a = uf_find(par, a);
        b = uf_find(par, b);
        if (a == b) return;
        if (a > b) { int t = a; a = b; b = t; }
        int old = atomicCAS(&par[b], b, a);
        if (old == b) return;
        b = old;
    }
    set_status(status, ST_TIMEOUT);
}

__device__ __forceinline__ int first_slot(int node, int leafBase)
{
    while (node < leafBase) node <<= 1;
    return (node - leafBase) * SKID_LEAF;
}

__global__ void uf_init(int *par, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        par[i] = i;
}

// Mark cliques (hi.w = 1) and pre-link them.
__global__ void clique_kernel(float4 *lo, float4 *hi, int leafBase, int n, float tau2, int *par,
                              unsigned *status)
{
    for (int node = blockIdx.x * blockDim.x + threadIdx.x + 1; node < 2 * leafBase;
         node += gridDim.x * blockDim.x) {
        float4 l = lo[node], h = hi[node];
        float dx = h.x - l.x, dy = h.y - l.y, dz = h.z - l.z;
        bool empty = !(dx >= 0.0f);
        float diag2 = dx * dx + dy * dy + dz * dz;
        bool clique = !empty && diag2 * (1.0f + 1e-5f) < tau2;
        h.w = clique ? 1.0f : 0.0f;
        hi[node] = h;
        if (!clique) continue;
        if (node >= leafBase) {
            int b = (node - leafBase) * SKID_LEAF, e = min(b + SKID_LEAF, n);
            for (int j = b + 1; j < e; ++j) uf_union(par, b, j, status);
        } else {
            int a = first_slot(2 * node, leafBase), c = first_slot(2 * node + 1, leafBase);
            if (a < n && c < n) uf_union(par, a, c, status);
        }
    }
}

// One warp per leaf of queries; each pair is linked from its lower slot, so
// subtrees wholly below the query leaf are skipped.  The last 2^subShift
// leaves under a node are tested one per lane against the query leaf's box;
// at a visited leaf, only candidates above the first query slot within tau
// of the query box are compacted and tested.  A clique node (box diagonal
// below tau) is skipped by a lane already in its component.
__global__ void __launch_bounds__(F_WARPS * 32, 8)
link_kernel(TreeView t, float tau2, float3 L, float3 hL, bool per, int subShift, int *par,
            int *work, unsigned *status)
{
    __shared__ float4 cand[F_WARPS][SKID_LEAF];
    __shared__ int cslot[F_WARPS][SKID_LEAF];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int rootLo = t.leafBase >> subShift;
    const int logLeafBase = 31 - __clz(t.leafBase);
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
        const int own = t.leafBase + leaf;
        const float4 qlo = t.lo[own], qhi = t.hi[own];
        int cp = 1;
        for (;;) {
            // the last leaf under cp (its subtree is skipped when below ours)
            const int last = ((cp + 1) << (logLeafBase - (31 - __clz(cp)))) - 1;
            if (last >= own) {
                if (cp >= rootLo) {
                    const int first = cp << subShift;
                    bool pass = false;
                    if (lane < (1 << subShift) && first + lane >= own &&
                        first + lane - t.leafBase < t.nLeaf)
                        pass = boxbox_lb(qlo, qhi, t.lo[first + lane], t.hi[first + lane], L, per) < tau2;
                    for (unsigned lm = __ballot_sync(SKID_FULL, pass); lm; lm &= lm - 1) {
                        const int node = first + __ffs(lm) - 1;
                        float4 blo = t.lo[node], bhi = t.hi[node];
                        bool want = valid && box_lb(q, blo, bhi, L, per) < tau2;
                        if (want && bhi.w != 0.0f) {
                            int f = first_slot(node, t.leafBase);
                            if (uf_find(par, qi) == uf_find(par, f)) want = false;
                        }
                        if (!__any_sync(SKID_FULL, want)) continue;
                        const int cb = (node - t.leafBase) * SKID_LEAF;
                        const int cnt = min(SKID_LEAF, t.n - cb);
                        bool rel = false;
                        float4 c4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (lane < cnt && cb + lane > base) {
                            c4 = t.pos[cb + lane];
                            rel = box_lb(make_float3(c4.x, c4.y, c4.z), qlo, qhi, L, per) < tau2;
                        }
                        const unsigned R = __ballot_sync(SKID_FULL, rel);
                        const int nR = __popc(R);
                        __syncwarp();
                        if (rel) {
                            const int k = __popc(R & ((1u << lane) - 1u));
                            cand[w][k] = c4;
                            cslot[w][k] = cb + lane;
                        }
                        __syncwarp();
                        if (!want) continue;
                        int cx = img_class(q.x, blo.x, bhi.x, hL.x);
                        int cy = img_class(q.y, blo.y, bhi.y, hL.y);
                        int cz = img_class(q.z, blo.z, bhi.z, hL.z);
                        bool noshift = (cx == 0) & (cy == 0) & (cz == 0);
                        for (int j = 0; j < nR; ++j) {
                            const int sj = cslot[w][j];
                            if (sj <= qi) continue;
                            float4 c = cand[w][j];
                            float d;
                            if (noshift) {
                                d = d2of(fsub(q.x, c.x), fsub(q.y, c.y), fsub(q.z, c.z));
                            } else {
                                float d1 = d2of(img_dx(q.x, c.x, L.x, hL.x), img_dx(q.y, c.y, L.y, hL.y),
                                                img_dx(q.z, c.z, L.z, hL.z));
                                float d2v = d2of(img_dx(c.x, q.x, L.x, hL.x), img_dx(c.y, q.y, L.y, hL.y),
                                                 img_dx(c.z, q.z, L.z, hL.z));
                                d = fminf(d1, d2v);
                            }
                            if (d < tau2) uf_union(par, qi, sj, status);
                        }
                    }
                } else {
                    float4 blo = t.lo[cp], bhi = t.hi[cp];
                    bool want = valid && box_lb(q, blo, bhi, L, per) < tau2;
                    if (want && bhi.w != 0.0f) {
                        int f = first_slot(cp, t.leafBase);
                        if (uf_find(par, qi) == uf_find(par, f)) want = false;
                    }
                    if (__any_sync(SKID_FULL, want)) { cp <<= 1; continue; }
                }
            }
            cp = next_node(cp);
            if (cp == 1) break;
        }
    }
}

// label -> smallest member iOrder per root
__global__ void root_min_iorder(int *par, int n, const uint32_t *__restrict__ perm,
                                const int *__restrict__ mio, int *__restrict__ minio)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int r = uf_find(par, i);
        par[i] = r;
        atomicMin(&minio[r], mio[perm[i]]);
    }
}

__global__ void mark_roots(const int *__restrict__ par, const int *__restrict__ minio, int n,
                           int *__restrict__ flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (par[i] == i) flag[minio[i]] = 1;
}

__global__ void write_groups(const int *__restrict__ par, const int *__restrict__ minio,
                             const int *__restrict__ rank, int n, const uint32_t *__restrict__ perm,
                             const int *__restrict__ mio, int *__restrict__ grp)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int r = par[i];
        grp[mio[perm[i]]] = rank[minio[r]] + 1;
    }
}

__global__ void fill_int(int *p, int v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace

// FoF over np points (float4) whose iOrders are mio[perm-index]; writes
// group ids (1..) to grp[iOrder] and the group count to *d_ng.  Scratch:
// par[np], minio[np], flag/rank over the iOrder space [niorder].
cudaError_t fof_run(Tree &t, const float4 *pts, int np, const int *mio, int niorder, float tau,
                    float3 L, bool per, SortScratch &ss, DBuf<int> &par, DBuf<int> &minio,
                    DBuf<int> &flag, int *grp, int *d_ng, int *d_work, unsigned *d_status,
                    cudaStream_t st)
{
    cudaError_t e;
    if (np <= 0) return cudaMemsetAsync(d_ng, 0, sizeof(int), st);
    if ((e = tree_build(t, pts, np, false, ss, st))) return e;
    if ((e = dalloc(par, np)) || (e = dalloc(minio, np)) || (e = dalloc(flag, 2 * (size_t)niorder)))
        return e;
    float tau2 = tau * tau;
    float3 hL = make_float3(0.5f * L.x, 0.5f * L.y, 0.5f * L.z);
    uf_init<<<grid_for(np), 256, 0, st>>>(par.p, np); skid::note_launch();
    clique_kernel<<<grid_for(2 * t.leafBase), 256, 0, st>>>(t.lo.p, t.hi.p, t.leafBase, np, tau2,
                                                           par.p, d_status); skid::note_launch();
    if ((e = cudaMemsetAsync(d_work, 0, sizeof(int), st))) return e;
    int perSM = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, link_kernel, F_WARPS * 32, 0);
    if (perSM < 1) perSM = 1;
    int blocks = num_sms() * perSM;
    int need = (t.nLeaf + F_WARPS - 1) / F_WARPS;
    if (blocks > need) blocks = need;
    int subShift = 0;
    while (subShift < 5 && (2 << subShift) <= t.leafBase) ++subShift;
    link_kernel<<<blocks, F_WARPS * 32, 0, st>>>(t.view(), tau2, L, hL, per, subShift, par.p, d_work,
                                                 d_status); skid::note_launch();
    fill_int<<<grid_for(np), 256, 0, st>>>(minio.p, 0x7fffffff, np); skid::note_launch();
    root_min_iorder<<<grid_for(np), 256, 0, st>>>(par.p, np, t.perm.p, mio, minio.p); skid::note_launch();
    int *fl = flag.p, *rank = flag.p + niorder;
    if ((e = cudaMemsetAsync(fl, 0, niorder * sizeof(int), st))) return e;
    mark_roots<<<grid_for(np), 256, 0, st>>>(par.p, minio.p, np, fl); skid::note_launch();
    if ((e = scan_exclusive(fl, rank, niorder, d_ng, ss, st))) return e;
    write_groups<<<grid_for(np), 256, 0, st>>>(par.p, minio.p, rank, np, t.perm.p, mio, grp); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
