// skid_knn_ball2_noalloc: the k-nearest-neighbour ball radii without any
// device allocation.
//
// Some callers cannot call cudaMalloc: a host framework that owns the device
// allocator and requires every device byte to come from its own pool, or a
// latency-critical loop where cudaMalloc/cudaFree's implicit device
// synchronisation is not acceptable.  This entry point takes device pointers
// for its input and output and keeps every intermediate (sort keys, the
// tree, the per-point results before un-permuting) in one file-scope
// __device__ array of fixed size.  Limits: at most SKID_NOALLOC_MAX_POINTS
// points and SKID_NOALLOC_MAX_K neighbours (the per-lane heaps then fit in
// shared memory); larger requests are refused with SKID_ETOOLARGE.
//
// The array lives on every GPU that loads the library until the process
// exits.  Host code cannot use the array's name as a device address, so the
// first call on each device looks the address up with cudaGetSymbolAddress
// (with that device current) and caches it; make that first call before any
// stream capture.  All calls share the array and it keeps the last call's
// contents: every buffer is rewritten or cleared before use, and two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it.  A call that fails with SKID_ECUDA has consumed the
// device's last-error state (cudaGetLastError), including an error that
// something else on this thread left pending.
#include <cfloat>
#include <mutex>

#include "../../include/skid_gpu.h"
#include "internal.h"

namespace skid {

namespace {

constexpr int NA_MAXN = SKID_NOALLOC_MAX_POINTS;
constexpr int NA_MAXK = SKID_NOALLOC_MAX_K;
constexpr int NA_LEAFBASE = (NA_MAXN + SKID_LEAF - 1) / SKID_LEAF;   // power of two
constexpr int NA_NODES = 2 * NA_LEAFBASE;
constexpr int NA_TILES = (NA_MAXN + 4095) / 4096;                   // radix-sort tiles

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets inside the scratch array
constexpr size_t OFF_P4 = 0;
constexpr size_t OFF_K0 = align256(OFF_P4 + sizeof(float4) * NA_MAXN);
constexpr size_t OFF_K1 = align256(OFF_K0 + sizeof(uint64_t) * NA_MAXN);
constexpr size_t OFF_V0 = align256(OFF_K1 + sizeof(uint64_t) * NA_MAXN);
constexpr size_t OFF_V1 = align256(OFF_V0 + sizeof(uint32_t) * NA_MAXN);
constexpr size_t OFF_HIST = align256(OFF_V1 + sizeof(uint32_t) * NA_MAXN);
constexpr size_t OFF_BLK = align256(OFF_HIST + sizeof(uint32_t) * 256 * NA_TILES);
constexpr size_t OFF_BOX = align256(OFF_BLK + sizeof(int) * 64);
constexpr size_t OFF_TPOS = align256(OFF_BOX + sizeof(unsigned) * 8);
constexpr size_t OFF_PERM = align256(OFF_TPOS + sizeof(float4) * NA_MAXN);
constexpr size_t OFF_LO = align256(OFF_PERM + sizeof(uint32_t) * NA_MAXN);
constexpr size_t OFF_HI = align256(OFF_LO + sizeof(float4) * NA_NODES);
constexpr size_t OFF_FLAG = align256(OFF_HI + sizeof(float4) * NA_NODES);
constexpr size_t OFF_B2 = align256(OFF_FLAG + sizeof(int) * NA_NODES);
constexpr size_t OFF_WORK = align256(OFF_B2 + sizeof(float) * NA_MAXN);
constexpr size_t OFF_GLOB = align256(OFF_WORK + sizeof(int) * 64);
constexpr size_t NA_BYTES = align256(OFF_GLOB + sizeof(uint32_t) * SORT_GLOB_WORDS);

static_assert((NA_LEAFBASE & (NA_LEAFBASE - 1)) == 0, "leaf count must be a power of two");
static_assert(NA_BYTES < (8u << 20), "scratch must stay modest");

__device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_mu;
unsigned char *g_addr[SKID_MAX_DEVICES] = {};

__global__ void na_xyz_to_pos4(const float *__restrict__ xyz, int n, float4 *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = make_float4(xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2],
                             0.0f);
}

__global__ void na_unsort(const uint32_t *__restrict__ perm, const float *__restrict__ in, int n,
                          float *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[perm[i]] = in[i];
}

template <typename T>
DBuf<T> view(unsigned char *base, size_t off, size_t count)
{
    DBuf<T> b;
    b.p = reinterpret_cast<T *>(base + off);
    b.n = count;
    return b;
}

// Scratch address on the current device (looked up once per device).
int scratch_address(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SKID_MAX_DEVICES) {
        cudaGetLastError();
        return SKID_ENODEV;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SKID_ECUDA;
        }
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return 0;
}

}  // namespace

}  // namespace skid

using namespace skid;

extern "C" int skid_knn_ball2_noalloc(const float *d_pos, int n, int k, const float period[3],
                                      float *d_ball2, void *stream)
{
    if (n < 0 || !period || (n > 0 && (!d_pos || !d_ball2))) return SKID_EINVAL;
    if (n > NA_MAXN || k > NA_MAXK) return SKID_ETOOLARGE;
    if (n == 0) return 0;
    if (k < 1 || k > n) return SKID_EINVAL;
    // the per-lane heaps must fit in shared memory (the kNN launcher would
    // otherwise put them in allocated global memory)
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return SKID_ENODEV;
    }
    if ((size_t)SKID_LEAF * sizeof(float4) + (size_t)k * 32 * sizeof(float) > (size_t)optin)
        return SKID_ETOOLARGE;
    unsigned char *base = nullptr;
    if (int rc = scratch_address(&base)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SortScratch ss;
    ss.k0 = view<uint64_t>(base, OFF_K0, NA_MAXN);
    ss.k1 = view<uint64_t>(base, OFF_K1, NA_MAXN);
    ss.v0 = view<uint32_t>(base, OFF_V0, NA_MAXN);
    ss.v1 = view<uint32_t>(base, OFF_V1, NA_MAXN);
    ss.hist = view<uint32_t>(base, OFF_HIST, 256 * (size_t)NA_TILES);
    ss.glob = view<uint32_t>(base, OFF_GLOB, SORT_GLOB_WORDS);
    ss.blk = view<int>(base, OFF_BLK, 64);
    ss.box = view<unsigned>(base, OFF_BOX, 8);
    Tree t;
    t.pos = view<float4>(base, OFF_TPOS, NA_MAXN);
    t.perm = view<uint32_t>(base, OFF_PERM, NA_MAXN);
    t.lo = view<float4>(base, OFF_LO, NA_NODES);
    t.hi = view<float4>(base, OFF_HI, NA_NODES);
    t.flag = view<int>(base, OFF_FLAG, NA_NODES);
    DBuf<float4> p4 = view<float4>(base, OFF_P4, NA_MAXN);
    float *b_sorted = reinterpret_cast<float *>(base + OFF_B2);
    int *d_work = reinterpret_cast<int *>(base + OFF_WORK);
    DBuf<float> no_heap;   // never used: the heaps fit in shared memory (checked above)
    float3 L = make_float3(period[0], period[1], period[2]);
    bool per = period[0] < 0.25f * FLT_MAX;
    na_xyz_to_pos4<<<grid_for(n), 256, 0, st>>>(d_pos, n, p4.p); note_launch();
    cudaError_t e = tree_build(t, p4.p, n, false, ss, st);
    if (!e) e = knn_ball2(t, k, L, per, b_sorted, d_work, no_heap, st);
    if (!e) {
        na_unsort<<<grid_for(n), 256, 0, st>>>(t.perm.p, b_sorted, n, d_ball2); note_launch();
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SKID_ECUDA;
    }
    return 0;
}
