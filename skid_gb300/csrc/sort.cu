// Stable LSD radix sort (8-bit digits, one sweep per digit) and device-wide
// exclusive scan.
//
// The sort reads the keys once up front to count every digit position's
// histogram (one kernel for all passes), turns them into global digit
// offsets (one small kernel), then makes one kernel launch per 8-bit pass.
// A pass takes tiles of 4096 keys (each of 8 warps ranks 512 contiguous
// keys with warp match, so tile order = input order) in the order blocks
// start (a tile counter), so a tile's predecessors are always already
// running: it counts its digits, publishes them, and finds the keys of each
// digit before it by decoupled look-back over the predecessors' published
// counts (an aggregate, or an inclusive prefix that ends the walk), then
// scatters its keys stably.  Each look-back wait is bounded; one that runs
// out sets the caller's status word.

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
std::atomic<unsigned long long> g_alloc_epoch{0};
}  // namespace

unsigned long long alloc_epoch() { return g_alloc_epoch.load(); }
void bump_alloc_epoch() { ++g_alloc_epoch; }

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

// ---- one-sweep passes ----
constexpr int OS_WARPS = RS_WARPS;
constexpr int OS_MAXPASS = 8;
constexpr unsigned OS_AGG = 1u << 30;         // status: the tile's own digit count
constexpr unsigned OS_PRE = 2u << 30;         // status: inclusive prefix up to the tile
constexpr unsigned OS_VAL = (1u << 30) - 1u;
constexpr int OS_SPIN_LIMIT = 1 << 24;

// Digit histograms of every pass in one read of the keys, into glob[p*256+d].
__global__ void os_histogram(const uint64_t *__restrict__ keys, int n, const int *d_n, int passes,
                             uint32_t *__restrict__ glob)
{
    __shared__ uint32_t h[OS_MAXPASS * 256];
    if (d_n) n = min(n, *d_n);
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p * 256 + (int)((k >> (8 * p)) & 0xff)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
        if (h[i]) atomicAdd(&glob[i], h[i]);
}

// Histograms -> exclusive global offsets, one pass at a time (256 threads).
__global__ void os_offsets(uint32_t *glob, int passes)
{
    __shared__ uint32_t ws[8];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int p = 0; p < passes; ++p) {
        const uint32_t x = glob[p * 256 + t];
        uint32_t v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(SKID_FULL, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) ws[w] = v;
        __syncthreads();
        uint32_t before = 0;
        for (int j = 0; j < w; ++j) before += ws[j];
        glob[p * 256 + t] = before + v - x;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(RS_THREADS)
os_pass(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin,
        uint64_t *__restrict__ kout, uint32_t *__restrict__ vout, int n, const int *d_n, int shift,
        const uint32_t *__restrict__ goff, uint32_t *status, uint32_t *counter, unsigned *d_err)
{
    constexpr int WKEYS = RS_ROUNDS * 32;          // keys per warp, contiguous
    __shared__ uint32_t s_tile;
    __shared__ uint32_t wcnt[OS_WARPS][256];       // per-warp digit counts, then offsets
    __shared__ uint32_t run[256];                  // the tile's first output slot per digit
    if (d_n) n = min(n, *d_n);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
#pragma unroll
    for (int j = 0; j < OS_WARPS; ++j) wcnt[j][tid] = 0;
    __syncthreads();
    const int tile = (int)s_tile;
    const int base = tile * RS_TILE;
    if (base >= n) return;   // beyond the live keys (block-uniform)
    // warp w ranks keys [base + w WKEYS, base + (w+1) WKEYS) in 16 rounds of
    // 32: a key's place among its warp's keys of the same digit is the
    // count from earlier rounds plus its rank among equal digits this round
    const int wbase = base + w * WKEYS;
    const unsigned lt = (1u << lane) - 1u;
    uint64_t k[RS_ROUNDS];
    uint32_t v[RS_ROUNDS], loc[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbase + r * 32 + lane;
        const bool valid = i < n;
        k[r] = valid ? kin[i] : 0;
        v[r] = valid ? vin[i] : 0;
        const unsigned d = valid ? (unsigned)((k[r] >> shift) & 0xff) : 256u + lane;
        const unsigned peers = __match_any_sync(SKID_FULL, d);
        const unsigned before = valid ? wcnt[w][d] : 0u;
        __syncwarp();
        if (valid && (peers & lt) == 0) wcnt[w][d] = before + __popc(peers);
        __syncwarp();
        loc[r] = before + __popc(peers & lt);
    }
    __syncthreads();
    {
        // thread tid owns digit tid: the warps' exclusive offsets, the tile's
        // count, then publish and look back over the predecessors
        uint32_t c = 0;
#pragma unroll
        for (int j = 0; j < OS_WARPS; ++j) {
            const uint32_t x = wcnt[j][tid];
            wcnt[j][tid] = c;
            c += x;
        }
        uint32_t *mine = status + (size_t)tile * 256 + tid;
        uint32_t excl = 0;
        if (tile == 0) {
            atomicExch(mine, OS_PRE | c);
        } else {
            atomicExch(mine, OS_AGG | c);
            int t = tile - 1, spins = 0;
            for (;;) {
                const uint32_t sv = *(volatile const uint32_t *)(status + (size_t)t * 256 + tid);
                const uint32_t f = sv & ~OS_VAL;
                if (f == 0u) {
                    if (++spins > OS_SPIN_LIMIT) {
                        if (d_err) atomicOr(d_err, ST_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                excl += sv & OS_VAL;
                if (f == OS_PRE || t == 0) break;
                --t;
            }
            atomicExch(mine, OS_PRE | (excl + c));
        }
        run[tid] = goff[tid] + excl;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbase + r * 32 + lane;
        if (i < n) {
            const unsigned d = (unsigned)((k[r] >> shift) & 0xff);
            const unsigned off = run[d] + wcnt[w][d] + loc[r];
            kout[off] = k[r];
            vout[off] = v[r];
        }
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
    if (n <= 0 || bits <= 0) return cudaSuccess;
    const int passes = (bits + 7) / 8 < OS_MAXPASS ? (bits + 7) / 8 : OS_MAXPASS;
    const int nTiles = (n + RS_TILE - 1) / RS_TILE;
    cudaError_t e;
    if ((e = dalloc(s.hist, (size_t)256 * nTiles)) || (e = dalloc(s.glob, SORT_GLOB_WORDS)))
        return e;
    // glob: [p*256 + d] digit histograms -> offsets; [OS_MAXPASS*256 + p] tile counters
    if ((e = cudaMemsetAsync(s.glob.p, 0, SORT_GLOB_WORDS * sizeof(uint32_t), st))) return e;
    const int hblocks = nTiles < num_sms() * 2 ? nTiles : num_sms() * 2;
    os_histogram<<<hblocks, 512, 0, st>>>(s.k0.p, n, d_n, passes, s.glob.p); skid::note_launch();
    os_offsets<<<1, 256, 0, st>>>(s.glob.p, passes); skid::note_launch();
    for (int p = 0; p < passes; ++p) {
        if ((e = cudaMemsetAsync(s.hist.p, 0, (size_t)256 * nTiles * sizeof(uint32_t), st)))
            return e;
        os_pass<<<nTiles, RS_THREADS, 0, st>>>(s.k0.p, s.v0.p, s.k1.p, s.v1.p, n, d_n, 8 * p,
                                                s.glob.p + 256 * p, s.hist.p,
                                                s.glob.p + OS_MAXPASS * 256 + p, s.d_err); skid::note_launch();
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
