// Stable LSD radix sort (8-bit digits) and device-wide exclusive scan.
//
// Each sort pass: (1) per-tile digit histograms, (2) one exclusive scan over
// the digit-major count table, (3) a stable scatter that ranks keys inside
// the tile with warp match + per-warp digit counts.  Tiles are 4096 keys
// (256 threads x 16 rounds, round-major so tile order = input order).
#include <atomic>

#include "internal.h"

namespace skid {

namespace {
std::atomic<long long> g_launches{0};
thread_local bool g_capturing = false;
}  // namespace

void note_launch(int n)
{
    if (!g_capturing) g_launches += n;
}

long long launches_total() { return g_launches.load(); }

void set_capturing(bool on) { g_capturing = on; }

std::recursive_mutex &device_mutex()
{
    static std::recursive_mutex m;
    return m;
}

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void rs_histogram(const uint64_t *__restrict__ keys, int n, const int *d_n, int shift,
                             int nTiles, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t h[256];
    if (d_n) n = min(n, *d_n);   // live count known only on the device
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        int i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nTiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void rs_scatter(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                           uint64_t *__restrict__ kout, uint32_t *__restrict__ vout, int n,
                           const int *d_n, int shift, int nTiles, const uint32_t *__restrict__ offs)
{
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[RS_WARPS][256];
    if (d_n) n = min(n, *d_n);
    if ((int)blockIdx.x * RS_TILE >= n) return;   // tile beyond the live keys
    int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    run[tid] = offs[tid * nTiles + blockIdx.x];
    for (int j = 0; j < RS_WARPS; ++j) wcnt[j][tid] = 0;
    __syncthreads();
    int base = blockIdx.x * RS_TILE;
    unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        int i = base + r * RS_THREADS + tid;
        bool valid = i < n;
        uint64_t k = valid ? kin[i] : 0;
        uint32_t v = valid ? vin[i] : 0;
        unsigned d = valid ? (unsigned)((k >> shift) & 0xff) : 256u + lane;  // unique for invalid
        unsigned peers = __match_any_sync(SKID_FULL, d);
        unsigned rank = __popc(peers & lt);
        bool leader = (peers & lt) == 0;
        if (valid && leader) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned off = run[d] + rank;
            for (int j = 0; j < w; ++j) off += wcnt[j][d];
            kout[off] = k;
            vout[off] = v;
        }
        __syncthreads();
        {
            unsigned s = 0;
            for (int j = 0; j < RS_WARPS; ++j) { s += wcnt[j][tid]; wcnt[j][tid] = 0; }
            run[tid] += s;
        }
        __syncthreads();
    }
}

// ---- int scan: tile sums, then each tile from the sums before it ----
constexpr int SC_THREADS = 512;
constexpr int SC_ITEMS = 8;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__device__ __forceinline__ int block_excl_scan(int x, int *sh, int *total)
{
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(SKID_FULL, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        int s = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(SKID_FULL, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) sh[lane] = s;
    }
    __syncthreads();
    int before = (w ? sh[w - 1] : 0) + v - x;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void scan_tile_sums(const int *in, int n, int *blk)
{
    __shared__ int sh[32];
    int base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS;
    int s = 0;
#pragma unroll
    for (int j = 0; j < SC_ITEMS; ++j) s += (base + j < n) ? in[base + j] : 0;
    int tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) blk[blockIdx.x] = tot;
}

// Each block scans its tile from the sum of the tile sums before it (read
// here, so the scan takes two launches); block 0 also writes the total.
__global__ void scan_apply(const int *in, int *out, int n, const int *blk, int nb, int *d_total)
{
    __shared__ int sh[32];
    const int b = blockIdx.x;
    int pre = 0, all = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        int v = blk[k];
        all += v;
        if (k < b) pre += v;
    }
    int tot;
    block_excl_scan(pre, sh, &tot);
    pre = tot;
    block_excl_scan(all, sh, &tot);
    all = tot;
    int base = b * SC_TILE + threadIdx.x * SC_ITEMS;
    int v[SC_ITEMS];
    int s = 0;
#pragma unroll
    for (int j = 0; j < SC_ITEMS; ++j) {
        v[j] = (base + j < n) ? in[base + j] : 0;
        s += v[j];
    }
    int run = block_excl_scan(s, sh, &tot) + pre;
#pragma unroll
    for (int j = 0; j < SC_ITEMS; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (b == 0 && threadIdx.x == 0 && d_total) *d_total = all;
}

}  // namespace

int num_sms()
{
    // per device: a process may drive several GPUs (one context per thread)
    static std::atomic<int> sms[SKID_MAX_DEVICES];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SKID_MAX_DEVICES) {
        cudaGetLastError();
        dev = 0;
    }
    int v = sms[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            v <= 0) {
            cudaGetLastError();
            v = 1;
        }
        sms[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

cudaError_t radix_sort(SortScratch &s, int n, int bits, cudaStream_t st, const int *d_n)
{
    if (n <= 0) return cudaSuccess;
    int nTiles = (n + RS_TILE - 1) / RS_TILE;
    cudaError_t e = dalloc(s.hist, (size_t)256 * nTiles);
    if (e) return e;
    for (int shift = 0; shift < bits; shift += 8) {
        rs_histogram<<<nTiles, RS_THREADS, 0, st>>>(s.k0.p, n, d_n, shift, nTiles, s.hist.p); skid::note_launch();
        e = scan_exclusive((const int *)s.hist.p, (int *)s.hist.p, 256 * nTiles, nullptr, s, st);
        if (e) return e;
        rs_scatter<<<nTiles, RS_THREADS, 0, st>>>(s.k0.p, s.v0.p, s.k1.p, s.v1.p, n, d_n, shift, nTiles,
                                                  s.hist.p); skid::note_launch();
        std::swap(s.k0, s.k1);
        std::swap(s.v0, s.v1);
    }
    return cudaGetLastError();
}

cudaError_t scan_exclusive(const int *in, int *out, int n, int *d_total, SortScratch &s,
                           cudaStream_t st)
{
    if (n <= 0) {
        if (d_total) return cudaMemsetAsync(d_total, 0, sizeof(int), st);
        return cudaSuccess;
    }
    int nb = (n + SC_TILE - 1) / SC_TILE;
    if (nb > 512 * 16) return cudaErrorInvalidValue;  // > 33 M entries
    cudaError_t e = dalloc(s.blk, (size_t)nb);
    if (e) return e;
    scan_tile_sums<<<nb, SC_THREADS, 0, st>>>(in, n, s.blk.p); skid::note_launch();
    scan_apply<<<nb, SC_THREADS, 0, st>>>(in, out, n, s.blk.p, nb, d_total); skid::note_launch();
    return cudaGetLastError();
}

}  // namespace skid
