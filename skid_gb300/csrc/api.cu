// C ABI of libskidgpu (include/skid_gpu.h): the context and the pipeline
// stages of main.c:347-485 on one GB300.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "ctx.h"

using namespace skid;

namespace {

__global__ void pack_particles(const float *pos, const float *vel, const float *mass,
                               const float *soft, const float *temp, int n, float4 *pos4,
                               float4 *vel4, float *tempo)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        pos4[i] = make_float4(pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2],
                              mass[i]);
        vel4[i] = make_float4(vel[3 * (size_t)i], vel[3 * (size_t)i + 1], vel[3 * (size_t)i + 2],
                              soft[i]);
        tempo[i] = temp ? temp[i] : 0.0f;
    }
}

// Scatterers are whole type ranges (ScatterCriterion depends on type only,
// kd.c:600-627): map list index -> iOrder through up to three ranges.
__global__ void gather_ranges(Ranges r, const float4 *__restrict__ pos4, float4 *out, int *io)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r.n; i += gridDim.x * blockDim.x) {
        int j = i, k = 0;
        while (k < 2 && j >= r.len[k]) { j -= r.len[k]; ++k; }
        int o = r.start[k] + j;
        out[i] = pos4[o];
        io[i] = o;
    }
}

__global__ void permute_scat(const uint32_t *__restrict__ perm, const int *__restrict__ io_in,
                             const float *__restrict__ b_sorted, const float *__restrict__ rho_sorted,
                             int n, int *__restrict__ sidx, float *__restrict__ rho_io,
                             float *__restrict__ ball2_io, float *__restrict__ rho_final)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int o = io_in[perm[i]];
        sidx[i] = o;
        rho_io[o] = rho_sorted[i];
        rho_final[o] = rho_sorted[i];
        ball2_io[o] = b_sorted[i];
    }
}

__global__ void ball_aux(const float *__restrict__ b, int n, float4 *__restrict__ aux)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        aux[i] = make_float4(b[i], 0.0f, 0.0f, __uint_as_float(1u));
}

__global__ void fill_float(float *p, float v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

__global__ void iota_kernel(int *p, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// CutCriterion (kd.c:555-597).
__device__ __forceinline__ int ptype(int io, int nGas, int nDark, int n)
{
    return io < nGas ? 2 : (io < nGas + nDark ? 1 : (io < n ? 4 : 0));
}

__global__ void cut_criterion(const float4 *__restrict__ pos4, const float *__restrict__ rho,
                              const float *__restrict__ temp, int n, int nGas, int nDark,
                              int inType, float fDensMin, float fTempMax, float fMassMax, int bGD,
                              int bGO, int *__restrict__ flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int t = ptype(i, nGas, nDark, n);
        float m = pos4[i].w, r = rho[i], T = temp[i];
        int ok = 0;
        if (!(m > fMassMax)) {
            switch (inType) {
            case 1:
                ok = r >= fDensMin;
                break;
            case 2: case 3:
                if (bGD && t == 1 && r >= fDensMin) ok = 1;
                else ok = t == 2 && r >= fDensMin && T <= fTempMax;
                break;
            case 4: case 5:
                ok = t == 4;
                break;
            case 6: case 7:
                if (bGD && t == 1 && r >= fDensMin) ok = 1;
                else if (t == 2) ok = r >= fDensMin && T <= fTempMax;
                else ok = t == 4 && !bGO;
                break;
            }
        }
        flag[i] = ok;
    }
}

__global__ void compact_index(const int *__restrict__ flag, const int *__restrict__ pos, int n,
                              int *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flag[i]) out[pos[i]] = i;
}

__global__ void gather_by_index(const int *__restrict__ idx, const float4 *__restrict__ src, int n,
                                float4 *__restrict__ dst)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

__global__ void init_movers(const uint32_t *__restrict__ perm, const int *__restrict__ mio_in,
                            const float4 *__restrict__ pos4, int n, int *__restrict__ mio,
                            float4 *__restrict__ mpos, float4 *__restrict__ mold,
                            int *__restrict__ act)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int o = mio_in[perm[i]];
        float4 p = pos4[o];
        p.w = 0.0f;
        mio[i] = o;
        mpos[i] = p;
        mold[i] = p;
        act[i] = i;
    }
}

__global__ void moved_to_iorder(const float4 *__restrict__ mpos, const int *__restrict__ mio, int n,
                                float *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int o = mio[i];
        float4 p = mpos[i];
        out[3 * (size_t)o] = p.x;
        out[3 * (size_t)o + 1] = p.y;
        out[3 * (size_t)o + 2] = p.z;
    }
}

__global__ void pos4_to_xyz(const float4 *__restrict__ p, int n, float *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = p[i];
        out[3 * (size_t)i] = q.x;
        out[3 * (size_t)i + 1] = q.y;
        out[3 * (size_t)i + 2] = q.z;
    }
}

__global__ void unsort_floats(const uint32_t *__restrict__ perm, const float *__restrict__ in,
                              int n, float *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[perm[i]] = in[i];
}

__global__ void xyz_to_pos4(const float *__restrict__ xyz, int n, float4 *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = make_float4(xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2],
                             0.0f);
}

}  // namespace

// Largest float <= the double threshold t (so float compares match the
// reference's double compares, kd.c:724-727).
float skid::float_floor(double t)
{
    float f = (float)t;
    if ((double)f > t) f = nextafterf(f, -INFINITY);
    return f;
}

float3 skid_ctx::wrap_hi() const
{
    return make_float3(float_floor((double)par.center[0] + 0.5 * (double)par.period[0]),
                       float_floor((double)par.center[1] + 0.5 * (double)par.period[1]),
                       float_floor((double)par.center[2] + 0.5 * (double)par.period[2]));
}

float3 skid_ctx::wrap_lo() const
{
    return make_float3(float_floor((double)par.center[0] - 0.5 * (double)par.period[0]),
                       float_floor((double)par.center[1] - 0.5 * (double)par.period[1]),
                       float_floor((double)par.center[2] - 0.5 * (double)par.period[2]));
}

// ---------------------------------------------------------------------
// context helpers

int skid_ctx::fail(int code)
{
    if (!last_error) last_error = code;
    return code;
}

int skid_ctx::fail_cuda(cudaError_t e)
{
    if (!last_cuda) last_cuda = (int)e;
    cudaGetLastError();
    return fail(SKID_ECUDA);
}

int skid_ctx::sync_check()
{
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e);
    unsigned s = 0;
    e = cudaMemcpyAsync(&s, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e);
    if (s & ST_TIMEOUT) return fail(SKID_ETIMEOUT);
    if (s & ST_OVERFLOW) return fail(SKID_EOVERFLOW);
    if (s) return fail(SKID_ECUDA);
    return 0;
}

int skid_ctx::read_int(const int *d, int *h)
{
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return fail_cuda(e);
    return sync_check();
}

void skid_ctx::timer_start()
{
    cudaEventRecord(ev0, st);
}

float skid_ctx::timer_stop()
{
    cudaEventRecord(ev1, st);
    cudaEventSynchronize(ev1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    return ms;
}

FieldArgs skid_ctx::field_args(float fStep, bool initial, float *acc_out)
{
    (void)initial;
    FieldArgs a;
    a.cpos = C.cpos.p;
    a.ccoef = C.ccoef.p;
    a.blo = ctree.blo.p;
    a.bhi = ctree.bhi.p;
    a.leafBase = ctree.leafBase;
    a.logLeafBase = 0;
    while ((2 << a.logLeafBase) <= a.leafBase) ++a.logLeafBase;
    a.d_nC = C.d_n;
    a.mpos = M.mpos.p;
    a.act = M.act.p;
    a.d_nA = M.d_nA;
    a.fStep = fStep;
    a.period = L;
    a.wrapHi = wrap_hi();
    a.wrapLo = wrap_lo();
    a.acc_out = acc_out;
    a.touched = C.touched.p;
    a.d_work = d_scal + SC_WORK;
    a.d_status = d_status;
    a.stats = field_stats_on ? d_fstats : nullptr;
    a.part_acc = split_acc.p;
    a.part_cnt = split_cnt.p;
    a.G = movers_per_warp();
    return a;
}

// One move pass: field + move, cut, refit.  Stream-ordered, no host sync.
// `slot` picks the event pair that times this step's field kernel.
int skid_ctx::enqueue_step(float fStep, bool initial, bool nocut, int slot, int G, bool compact)
{
    skid_ctx *ctx = this;
    FieldArgs a = field_args(fStep, initial, nullptr);
    a.G = G;
    // while capturing, external records make the events real timing nodes of
    // the outer-iteration graph (a plain record would only order the capture)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs));
    unsigned evflags = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
    CK(cudaEventRecordWithFlags(fev[2 * slot], st, evflags));
    if (opt_field_unfused) {
        if (unfused_acc.n < 3 * (size_t)nMove) return fail(SKID_ESTATE);
        a.fStep = 0.0f;
        a.acc_out = unfused_acc.p;
        CK(field_move(a, nMove, st));
        CK(move_movers(a, unfused_acc.p, fStep, nMove, st));
    } else {
        CK(field_move(a, nMove, st));
    }
    CK(cudaEventRecordWithFlags(fev[2 * slot + 1], st, evflags));
    CK(scatter_cut(C, initial, nocut, rho_final.p, M.d_nA, d_fbytes, compact, st));
    CK(tree_refit(ctree, C.cpos.p, nullptr, C.d_n, st, true, C.d_dirty));
    // between prunes, re-sort the active movers while they are many (16 or
    // more per warp): the warps' boxes stay tight as the movers drift
    if (!compact && G >= 16) CK(mover_resort(M, mkey_lo, mkey_inv, ss, st, slot_bound(G), opt_curve & 1));
    return 0;
}

void skid_ctx::collect_field_times(int nslots)
{
    for (int i = 0; i < nslots; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, fev[2 * i], fev[2 * i + 1]) == cudaSuccess) tim.field_ms += ms;
        else cudaGetLastError();
    }
}

// ---------------------------------------------------------------------
// C ABI

// Move field at nm explicit positions from the current live copies, left in
// probe_acc (the body of skid_field and skid_field_adjoint).
static int field_probe(skid_ctx *ctx, int nm, const float *mpos)
{
    cudaStream_t st = ctx->st;
    DBuf<float> &xyz = ctx->probe_f;
    DBuf<float4> &p4 = ctx->probe_p4;
    DBuf<int> &act = ctx->probe_i;
    if (dalloc(xyz, 3 * (size_t)nm) || dalloc(p4, nm) || dalloc(act, nm + 2) ||
        dalloc(ctx->probe_acc, 3 * (size_t)nm))
        return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(xyz.p, mpos, 3 * (size_t)nm * sizeof(float), cudaMemcpyHostToDevice, st));
    xyz_to_pos4<<<grid_for(nm), 256, 0, st>>>(xyz.p, nm, p4.p); skid::note_launch();
    iota_kernel<<<grid_for(nm), 256, 0, st>>>(act.p, nm); skid::note_launch();
    CK(cudaMemcpyAsync(act.p + nm, &nm, sizeof(int), cudaMemcpyHostToDevice, st));
    FieldArgs a = ctx->field_args(0.0f, false, ctx->probe_acc.p);
    a.mpos = p4.p;
    a.act = act.p;
    a.d_nA = act.p + nm;
    a.G = ctx->opt_G ? ctx->opt_G : 32;   // a forced movers-per-warp applies here too
    a.stats = nullptr;
    a.part_acc = nullptr;   // a probe walks each position in one warp
    a.part_cnt = nullptr;
    a.touched = ctx->probe_touched();
    if (!a.touched) return ctx->fail(SKID_ENOMEM);
    CK(field_move(a, nm, st));
    return 0;
}

// dL/dy = w * grad rho_f = -w * (move field)
__global__ void scale_field(float *acc, const float *__restrict__ w, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = -w[i];
        acc[3 * (size_t)i] *= s;
        acc[3 * (size_t)i + 1] *= s;
        acc[3 * (size_t)i + 2] *= s;
    }
}

extern "C" {

const char *skid_strerror(int code)
{
    switch (code) {
    case SKID_OK: return "ok";
    case SKID_EINVAL: return "invalid argument";
    case SKID_ENOMEM: return "out of memory";
    case SKID_ECUDA: return "CUDA runtime error";
    case SKID_ETIMEOUT: return "bounded device wait ran out";
    case SKID_EOVERFLOW: return "internal capacity exceeded";
    case SKID_ENODEV: return "no usable sm_103 device";
    case SKID_ESTATE: return "call made in the wrong pipeline state";
    case SKID_ETOOLARGE: return "request exceeds a fixed capacity";
    }
    return "unknown error";
}

int skid_last_error(const skid_ctx *ctx) { return ctx ? ctx->last_error : SKID_EINVAL; }

const char *skid_last_cuda_error(const skid_ctx *ctx)
{
    if (!ctx || !ctx->last_cuda) return "none";
    return cudaGetErrorString((cudaError_t)ctx->last_cuda);
}

int skid_create(skid_ctx **pctx, const skid_params *par)
{
    if (!pctx || !par) return SKID_EINVAL;
    *pctx = nullptr;
    if (par->nSmooth < 1) return SKID_EINVAL;
    // a period is positive (FLT_MAX: no period along that axis); NaN fails too
    for (int d = 0; d < 3; ++d)
        if (!(par->period[d] > 0.0f)) return SKID_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= par->device || par->device < 0) {
        cudaGetLastError();
        return SKID_ENODEV;
    }
    if (cudaSetDevice(par->device) != cudaSuccess) return SKID_ENODEV;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, par->device) != cudaSuccess) return SKID_ENODEV;
    if (prop.major < 10) return SKID_ENODEV;
    skid_ctx *ctx = new (std::nothrow) skid_ctx();
    if (!ctx) return SKID_ENOMEM;
    ctx->par = *par;
    ctx->L = make_float3(par->period[0], par->period[1], par->period[2]);
    ctx->hL = make_float3(0.5f * par->period[0], 0.5f * par->period[1], 0.5f * par->period[2]);
    ctx->per = par->period[0] < 0.25f * FLT_MAX;
    bool ok;
    {
        std::lock_guard<std::recursive_mutex> lk(device_mutex());
        ok = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) == cudaSuccess &&
             cudaMalloc((void **)&ctx->d_scal, SC_COUNT * sizeof(int)) == cudaSuccess &&
             cudaMalloc((void **)&ctx->d_fbytes, 2 * sizeof(double)) == cudaSuccess &&
             cudaEventCreate(&ctx->ev0) == cudaSuccess && cudaEventCreate(&ctx->ev1) == cudaSuccess;
        for (cudaEvent_t &e : ctx->fev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    }
    if (!ok) {
        delete ctx;
        return SKID_ENOMEM;
    }
    cudaMemsetAsync(ctx->d_scal, 0, SC_COUNT * sizeof(int), ctx->st);
    cudaMemsetAsync(ctx->d_fbytes, 0, 2 * sizeof(double), ctx->st);
    cudaStreamSynchronize(ctx->st);
    ctx->d_status = (unsigned *)(ctx->d_scal + SC_STATUS);
    ctx->ss.d_err = ctx->d_status;
    ctx->C.d_n = ctx->d_scal + SC_NC;
    ctx->C.d_n2 = ctx->d_scal + SC_NC2;
    ctx->C.d_floor = (unsigned *)(ctx->d_scal + SC_FLOOR);
    ctx->C.d_dirty = ctx->d_scal + SC_DIRTY;
    ctx->C.d_done = ctx->d_scal + SC_DONE;
    ctx->M.d_nA = ctx->d_scal + SC_NA;
    ctx->M.d_nA2 = ctx->d_scal + SC_NA2;
    *pctx = ctx;
    return 0;
}

int skid_destroy(skid_ctx *ctx)
{
    if (!ctx) return SKID_EINVAL;
    cudaSetDevice(ctx->par.device);
    cudaStreamSynchronize(ctx->st);
    delete ctx;
    return 0;
}

// Total |mass| (FP64) and smallest softening of the input, in a fixed order:
// block b reduces its contiguous chunk (thread-strided, then a fixed tree),
// and one warp adds the block partials in block order.
constexpr int MS_BLOCKS = 128;
constexpr int MS_THREADS = 256;

__global__ void __launch_bounds__(MS_THREADS)
mass_soft_partials(const float *__restrict__ mass, const float *__restrict__ soft, int n,
                   double *__restrict__ out)
{
    __shared__ double sm[MS_THREADS];
    __shared__ float ss[MS_THREADS];
    const int chunk = (n + MS_BLOCKS - 1) / MS_BLOCKS;
    const int b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    double m = 0.0;
    float e = FLT_MAX;
    for (int i = b0 + threadIdx.x; i < b1; i += MS_THREADS) {
        m += fabs((double)mass[i]);
        e = fminf(e, soft[i]);
    }
    sm[threadIdx.x] = m;
    ss[threadIdx.x] = e;
    __syncthreads();
    for (int h = MS_THREADS / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            sm[threadIdx.x] += sm[threadIdx.x + h];
            ss[threadIdx.x] = fminf(ss[threadIdx.x], ss[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 + 2 * blockIdx.x] = sm[0];
        out[3 + 2 * blockIdx.x] = (double)ss[0];
    }
}

__global__ void mass_soft_total(double *out)
{
    if (threadIdx.x != 0) return;
    double m = 0.0, e = (double)FLT_MAX;
    for (int b = 0; b < MS_BLOCKS; ++b) {
        m += out[2 + 2 * b];
        e = fmin(e, out[3 + 2 * b]);
    }
    out[0] = m;
    out[1] = e;
}

}  // extern "C"

namespace {

// Common first half of a particle upload: counts, pipeline reset, buffers.
int load_begin(skid_ctx *ctx, int nGas, int nDark, int nStar, double time)
{
    long long nn = (long long)nGas + nDark + nStar;
    // no particles, a negative count or more than 2^28: nothing to run
    if (nGas < 0 || nDark < 0 || nStar < 0 || nn <= 0 || nn > (1ll << 28))
        return ctx->fail(SKID_EINVAL);
    int n = (int)nn;
    cudaSetDevice(ctx->par.device);
    ctx->reset_pipeline();
    ctx->n = n;
    ctx->nGas = nGas;
    ctx->nDark = nDark;
    ctx->nStar = nStar;
    ctx->time = time;
    ctx->inType = (nDark ? 1 : 0) | (nGas ? 2 : 0) | (nStar ? 4 : 0);
    ctx->mass_total = 0.0;
    ctx->soft_min = ctx->soft_min_input = 0.0f;
    ctx->ms_pending = false;
    ctx->soft_changed = false;
    if (ctx->alloc_particles(n)) return ctx->fail(SKID_ENOMEM);
    if (n > 0 && dalloc(ctx->ms_dev, 2 * (size_t)MS_BLOCKS + 2)) return ctx->fail(SKID_ENOMEM);
    return 0;
}

// Common second half: the staged SoA arrays in ctx->raw (pos 3n, vel 3n,
// mass n, soft n, temp n) packed into the float4 records, the potential
// scale's reductions, and the per-particle outputs cleared.
int load_finish(skid_ctx *ctx, bool have_temp)
{
    const int n = ctx->n;
    float *d_raw = ctx->raw.p;
    const size_t n3 = 3 * (size_t)n;
    pack_particles<<<grid_for(n), 256, 0, ctx->st>>>(d_raw, d_raw + n3, d_raw + 2 * n3,
                                                     d_raw + 2 * n3 + n,
                                                     have_temp ? d_raw + 2 * n3 + 2 * (size_t)n : nullptr,
                                                     n, ctx->pos4.p, ctx->vel4.p, ctx->temp.p); skid::note_launch();
    CK(cudaGetLastError());
    // total |mass| and smallest softening for the potential scale (fixed order)
    mass_soft_partials<<<MS_BLOCKS, MS_THREADS, 0, ctx->st>>>(d_raw + 2 * n3, d_raw + 2 * n3 + n, n,
                                                             ctx->ms_dev.p); skid::note_launch();
    mass_soft_total<<<1, 32, 0, ctx->st>>>(ctx->ms_dev.p); skid::note_launch();
    ctx->ms_pending = true;
    fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->rho.p, 0.0f, n); skid::note_launch();
    fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->rho_final.p, 0.0f, n); skid::note_launch();
    fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->ball2.p, -1.0f, n); skid::note_launch();
    CK(cudaMemsetAsync(ctx->grp.p, 0, n * sizeof(int), ctx->st));
    ctx->stage = STAGE_LOADED;
    return ctx->sync_check();
}

// TIPSY particle records (kd.c:164-217; tipsydefs.h:6-37), one thread per
// particle: gas 12 words (mass pos vel rho temp hsmooth metals phi), dark 9
// (mass pos vel eps phi), star 11 (mass pos vel metals tform eps phi), in
// that order; XDR words are big-endian.  Writes the staged SoA arrays.
__global__ void unpack_tipsy(const uint32_t *__restrict__ w, int nGas, int nDark, int n, int swap,
                             float *__restrict__ pos, float *__restrict__ vel,
                             float *__restrict__ mass, float *__restrict__ soft,
                             float *__restrict__ temp)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        size_t off;
        int isoft, itemp = -1;
        if (i < nGas) {
            off = 12 * (size_t)i;
            isoft = 9;
            itemp = 8;
        } else if (i < nGas + nDark) {
            off = 12 * (size_t)nGas + 9 * (size_t)(i - nGas);
            isoft = 7;
        } else {
            off = 12 * (size_t)nGas + 9 * (size_t)nDark + 11 * (size_t)(i - nGas - nDark);
            isoft = 9;
        }
        auto word = [&](int k) {
            uint32_t v = __ldg(w + off + k);
            return __uint_as_float(swap ? __byte_perm(v, 0, 0x0123) : v);
        };
        mass[i] = word(0);
        pos[3 * (size_t)i] = word(1);
        pos[3 * (size_t)i + 1] = word(2);
        pos[3 * (size_t)i + 2] = word(3);
        vel[3 * (size_t)i] = word(4);
        vel[3 * (size_t)i + 1] = word(5);
        vel[3 * (size_t)i + 2] = word(6);
        soft[i] = word(isoft);
        temp[i] = itemp >= 0 ? word(itemp) : 0.0f;
    }
}

}  // namespace

extern "C" {

int skid_set_particles(skid_ctx *ctx, int nGas, int nDark, int nStar, double time,
                       const float *pos, const float *vel, const float *mass, const float *soft,
                       const float *temp)
{
    if (!ctx || nGas < 0 || nDark < 0 || nStar < 0 || !pos || !vel || !mass || !soft)
        return SKID_EINVAL;
    if (int rc = load_begin(ctx, nGas, nDark, nStar, time)) return rc;
    const int n = ctx->n;
    if (n == 0) { ctx->stage = STAGE_LOADED; return 0; }
    // staging: raw host arrays -> device, then pack to float4 records
    float *d_raw = ctx->raw.p;
    size_t n3 = 3 * (size_t)n;
    CK(cudaMemcpyAsync(d_raw, pos, n3 * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_raw + n3, vel, n3 * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_raw + 2 * n3, mass, n * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_raw + 2 * n3 + n, soft, n * sizeof(float), cudaMemcpyHostToDevice,
                       ctx->st));
    if (temp)
        CK(cudaMemcpyAsync(d_raw + 2 * n3 + 2 * (size_t)n, temp, n * sizeof(float),
                           cudaMemcpyHostToDevice, ctx->st));
    return load_finish(ctx, temp != nullptr);
}

int skid_set_tipsy(skid_ctx *ctx, int nGas, int nDark, int nStar, double time, int bStandard,
                   const void *records, size_t bytes)
{
    if (!ctx || nGas < 0 || nDark < 0 || nStar < 0) return SKID_EINVAL;
    const size_t want = 4 * (12 * (size_t)nGas + 9 * (size_t)nDark + 11 * (size_t)nStar);
    if (bytes != want || (want && !records)) return ctx->fail(SKID_EINVAL);
    if (int rc = load_begin(ctx, nGas, nDark, nStar, time)) return rc;
    const int n = ctx->n;
    if (n == 0) { ctx->stage = STAGE_LOADED; return 0; }
    if (dalloc(ctx->tipsy_raw, want / 4)) return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(ctx->tipsy_raw.p, records, want, cudaMemcpyHostToDevice, ctx->st));
    const uint32_t one = 1;
    const bool little = *reinterpret_cast<const unsigned char *>(&one) == 1;
    const int swap = (bStandard != 0) == little;   // XDR is big-endian
    float *d_raw = ctx->raw.p;
    const size_t n3 = 3 * (size_t)n;
    unpack_tipsy<<<grid_for(n), 256, 0, ctx->st>>>(ctx->tipsy_raw.p, nGas, nDark, n, swap, d_raw,
                                                   d_raw + n3, d_raw + 2 * n3, d_raw + 2 * n3 + n,
                                                   d_raw + 2 * n3 + 2 * (size_t)n); skid::note_launch();
    return load_finish(ctx, true);
}

int skid_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr) return SKID_EINVAL;
    *ptr = nullptr;
    if (cudaMallocHost(ptr, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return SKID_ENOMEM;
    }
    return 0;
}

int skid_host_free(void *ptr)
{
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return SKID_ECUDA;
    }
    return 0;
}

__global__ void restore_soft(float4 *vel4, const float *soft, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        vel4[i].w = soft[i];
}

int skid_restart(skid_ctx *ctx)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_LOADED) return ctx->fail(SKID_ESTATE);
    int n = ctx->n;
    if (ctx->ensure_mass_soft()) return ctx->fail(SKID_ECUDA);
    double mt = ctx->mass_total;
    float sm = ctx->soft_min_input;
    ctx->reset_pipeline();
    ctx->mass_total = mt;
    ctx->soft_min = sm;
    if (n > 0) {
        if (ctx->soft_changed) {
            restore_soft<<<grid_for(n), 256, 0, ctx->st>>>(ctx->vel4.p, ctx->soft_orig.p, n); skid::note_launch();
            ctx->soft_changed = false;
        }
        fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->rho.p, 0.0f, n); skid::note_launch();
        fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->rho_final.p, 0.0f, n); skid::note_launch();
        fill_float<<<grid_for(n), 256, 0, ctx->st>>>(ctx->ball2.p, -1.0f, n); skid::note_launch();
        CK(cudaMemsetAsync(ctx->grp.p, 0, n * sizeof(int), ctx->st));
    }
    ctx->stage = STAGE_LOADED;
    return ctx->sync_check();
}

int skid_scatter_active(skid_ctx *ctx, int bGasAndDark, int bGasOnly, int *nScatter)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_LOADED) return ctx->fail(SKID_ESTATE);
    // ScatterCriterion (kd.c:600-627) per type
    int t = ctx->inType;
    bool gas = false, dark = false, star = false;
    switch (t) {
    case 1: dark = true; break;
    case 2: case 3: gas = true; dark = bGasAndDark != 0; break;
    case 4: case 5: star = true; break;
    case 6: case 7:
        if (bGasAndDark) { gas = dark = star = true; }
        else { gas = true; star = !bGasOnly; }
        break;
    }
    Ranges r;
    r.n = 0;
    int k = 0;
    auto add = [&](bool on, int s, int l) {
        if (on && l > 0) { r.start[k] = s; r.len[k] = l; r.n += l; ++k; }
    };
    add(gas, 0, ctx->nGas);
    add(dark, ctx->nGas, ctx->nDark);
    add(star, ctx->nGas + ctx->nDark, ctx->nStar);
    for (; k < 3; ++k) { r.start[k] = 0; r.len[k] = 0; }
    ctx->ranges = r;
    ctx->nScatInit = r.n;
    if (nScatter) *nScatter = r.n;
    ctx->stage = STAGE_SCATTER;
    return 0;
}

int skid_density(skid_ctx *ctx, int *nExtraScat)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_SCATTER) return ctx->fail(SKID_ESTATE);
    int ns = ctx->nScatInit;
    if (ns < ctx->par.nSmooth) return ctx->fail(SKID_EINVAL);   // smooth1.c:12
    cudaSetDevice(ctx->par.device);
    if (ctx->alloc_scatterers(ns)) return ctx->fail(SKID_ENOMEM);
    cudaStream_t st = ctx->st;
    ctx->timer_start();
    Ranges r = ctx->ranges;
    gather_ranges<<<grid_for(ns), 256, 0, st>>>(r, ctx->pos4.p, ctx->spos0.p, ctx->sidx0.p); skid::note_launch();
    CK(cudaGetLastError());
    CK(tree_build(ctx->stree, ctx->spos0.p, ns, true, ctx->ss, st, ctx->opt_curve & 4));
    CK(knn_ball2(ctx->stree, ctx->par.nSmooth, ctx->L, ctx->per, ctx->sb2.p,
                 ctx->d_scal + SC_WORK, ctx->knn_heap, st));
    // node max fBall2 for the density gather
    ball_aux<<<grid_for(ns), 256, 0, st>>>(ctx->sb2.p, ns, ctx->saux.p); skid::note_launch();
    CK(tree_refit(ctx->stree, nullptr, ctx->saux.p, nullptr, st));
    CK(density_gather(ctx->stree, ctx->sb2.p, ctx->L, ctx->per, ctx->srho.p,
                      ctx->d_scal + SC_WORK, st));
    permute_scat<<<grid_for(ns), 256, 0, st>>>(ctx->stree.perm.p, ctx->sidx0.p, ctx->sb2.p,
                                               ctx->srho.p, ns, ctx->sidx.p, ctx->rho.p,
                                               ctx->ball2.p, ctx->rho_final.p); skid::note_launch();
    // move-phase copies (originals + periodic replicas) and their tree
    float3 blo = make_float3((float)((double)ctx->par.center[0] - 0.5 * (double)ctx->par.period[0]),
                             (float)((double)ctx->par.center[1] - 0.5 * (double)ctx->par.period[1]),
                             (float)((double)ctx->par.center[2] - 0.5 * (double)ctx->par.period[2]));
    float3 bhi = make_float3((float)((double)ctx->par.center[0] + 0.5 * (double)ctx->par.period[0]),
                             (float)((double)ctx->par.center[1] + 0.5 * (double)ctx->par.period[1]),
                             (float)((double)ctx->par.center[2] + 0.5 * (double)ctx->par.period[2]));
    int nc = 0;
    CK(build_copies(ctx->stree.pos.p, ctx->sb2.p, ctx->srho.p, ctx->sidx.p, ns, ctx->L, blo, bhi,
                    ctx->par.periodic != 0, ctx->C, ctx->ss, &nc, st, ctx->opt_curve & 2));
    CK(tree_shape(ctx->ctree, nc, true));
    CK(tree_refit(ctx->ctree, ctx->C.cpos.p, nullptr, ctx->C.d_n, st, true));
    ctx->nCopies = nc;
    int extra = nc - ns;
    if (int rc = ctx->sync_check()) return rc;
    ctx->nExtraScat = extra;
    ctx->tim.density_ms += ctx->timer_stop();
    if (nExtraScat) *nExtraScat = ctx->par.periodic ? extra : 0;
    ctx->stage = STAGE_DENSITY;
    return 0;
}

int skid_get_density(skid_ctx *ctx, float *rho, float *ball2)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    if (rho) CK(cudaMemcpyAsync(rho, ctx->rho.p, ctx->n * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
    if (ball2)
        CK(cudaMemcpyAsync(ball2, ctx->ball2.p, ctx->n * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
    return ctx->sync_check();
}

int skid_get_final_density(skid_ctx *ctx, float *rho)
{
    if (!ctx || !rho) return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    CK(cudaMemcpyAsync(rho, ctx->rho_final.p, ctx->n * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
    return ctx->sync_check();
}

int skid_init_move(skid_ctx *ctx, float fDensMin, float fTempMax, float fMassMax, int bGasAndDark,
                   int bGasOnly, int *nMove)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    int n = ctx->n;
    cudaStream_t st = ctx->st;
    if (ctx->alloc_movers(n)) return ctx->fail(SKID_ENOMEM);
    if (ctx->opt_field_unfused && dalloc(ctx->unfused_acc, 3 * (size_t)(n > 0 ? n : 1)))
        return ctx->fail(SKID_ENOMEM);
    cut_criterion<<<grid_for(n), 256, 0, st>>>(ctx->pos4.p, ctx->rho.p, ctx->temp.p, n, ctx->nGas,
                                               ctx->nDark, ctx->inType, fDensMin, fTempMax,
                                               fMassMax, bGasAndDark, bGasOnly, ctx->M.keep.p); skid::note_launch();
    CK(scan_exclusive(ctx->M.keep.p, ctx->M.kpos.p, n, ctx->M.d_nA, ctx->ss, st));
    compact_index<<<grid_for(n), 256, 0, st>>>(ctx->M.keep.p, ctx->M.kpos.p, n, ctx->M.act2.p); skid::note_launch();
    int nm = 0;
    if (int rc = ctx->read_int(ctx->M.d_nA, &nm)) return rc;
    ctx->nMove = nm;
    ctx->M.cap = nm > 0 ? nm : 1;   // prune passes and sorts run over this capacity
    // Hilbert order of the movers' starting positions keeps warps coherent.
    if (nm > 0) {
        gather_by_index<<<grid_for(nm), 256, 0, st>>>(ctx->M.act2.p, ctx->pos4.p, nm, ctx->M.mold.p); skid::note_launch();
        CK(curve_order(ctx->M.mold.p, nm, ctx->ss, st, ctx->opt_curve & 1));
        // key frame for the re-sorts at every prune: the periodic box, or the
        // movers' starting bounding box grown by half its size
        unsigned hb[6];
        CK(cudaMemcpyAsync(hb, ctx->ss.box.p, sizeof(hb), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        float lo3[3], hi3[3];
        for (int d = 0; d < 3; ++d) {
            unsigned u = hb[d], v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
            memcpy(&lo3[d], &v, 4);
            u = hb[3 + d];
            v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
            memcpy(&hi3[d], &v, 4);
            if (ctx->per) {
                lo3[d] = ctx->par.center[d] - 0.5f * ctx->par.period[d];
                hi3[d] = ctx->par.center[d] + 0.5f * ctx->par.period[d];
            } else {
                float g = 0.5f * (hi3[d] - lo3[d]);
                lo3[d] -= g;
                hi3[d] += g;
            }
        }
        float ext = fmaxf(fmaxf(hi3[0] - lo3[0], hi3[1] - lo3[1]), fmaxf(hi3[2] - lo3[2], 1e-30f));
        float sc = 2097151.0f / ext;
        ctx->mkey_lo = make_float3(lo3[0], lo3[1], lo3[2]);
        ctx->mkey_inv = make_float3(sc, sc, sc);
        init_movers<<<grid_for(nm), 256, 0, st>>>(ctx->ss.v0.p, ctx->M.act2.p, ctx->pos4.p, nm,
                                                   ctx->M.mio.p, ctx->M.mpos.p, ctx->M.mold.p,
                                                   ctx->M.act.p); skid::note_launch();
        CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(ctx->M.d_nA, &ctx->nMove, sizeof(int), cudaMemcpyHostToDevice, st));

    ctx->nActive = nm;
    if (nMove) *nMove = nm;
    ctx->stage = STAGE_MOVE;
    return ctx->sync_check();
}

int skid_move_step(skid_ctx *ctx, float fStep, int bInitial, int bNoCut, int *nScatter)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_MOVE) return ctx->fail(SKID_ESTATE);
    ctx->timer_start();
    bool ran = ctx->nMove > 0 || bInitial;
    if (ran) {
        int rc = ctx->enqueue_step(fStep, bInitial != 0, bNoCut != 0, 0, ctx->movers_per_warp());
        if (rc) return rc;
    }
    int live = 0;
    if (int rc = ctx->read_int(ctx->C.d_n2, &live)) return rc;
    if (ran) ctx->collect_field_times(1);
    float ms = ctx->timer_stop();
    if (ctx->stage >= STAGE_FOF) ctx->tim.micro_ms += ms;
    else ctx->tim.moving_ms += ms;
    if (nScatter) *nScatter = live;
    return 0;
}

int skid_prune_inactive(skid_ctx *ctx, float fCvg, int *nActive)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_MOVE) return ctx->fail(SKID_ESTATE);
    ctx->timer_start();
    CK(mover_prune(ctx->M, ctx->L, ctx->mkey_lo, ctx->mkey_inv, fCvg, ctx->ss, ctx->st, -1, ctx->opt_curve & 1));
    int na = 0;
    if (int rc = ctx->read_int(ctx->M.d_nA, &na)) return rc;
    ctx->tim.moving_ms += ctx->timer_stop();
    ctx->nActive = na;
    if (nActive) *nActive = na;
    return 0;
}

static int graph_slot(int G)
{
    return G == 32 ? 0 : G == 16 ? 1 : G == 8 ? 2 : G == 4 ? 3 : G == 64 ? 5 : 4;
}

int skid_move_iterate(skid_ctx *ctx, float fStep, float fCvg, int bNoCut, int *nActive,
                      int *nScatter)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_MOVE) return ctx->fail(SKID_ESTATE);
    cudaStream_t st = ctx->st;
    ctx->timer_start();
    int G = ctx->movers_per_warp();
    int gs = graph_slot(G);
    bool same = ctx->iter_graph[gs] && ctx->g_fStep[gs] == fStep && ctx->g_fCvg[gs] == fCvg &&
                ctx->g_nocut[gs] == (bNoCut != 0) && ctx->g_stats[gs] == ctx->field_stats_on &&
                ctx->g_bound[gs] >= ctx->nActive && ctx->g_key[gs] == ctx->graph_key();
    bool ran = false;
    if (!same) {
        if (ctx->iter_graph[gs]) {
            cudaGraphExecDestroy(ctx->iter_graph[gs]);
            ctx->iter_graph[gs] = nullptr;
        }
        if (!ctx->iter_eager_done) {
            // the first iteration runs eagerly; it sizes every scratch buffer
            for (int i = 0; i < PRUNE_STEPS; ++i)
                if (int rc = ctx->enqueue_step(fStep, false, bNoCut != 0, i, G, i == PRUNE_STEPS - 1))
                    return rc;
            CK(mover_prune(ctx->M, ctx->L, ctx->mkey_lo, ctx->mkey_inv, fCvg, ctx->ss, st, -1, ctx->opt_curve & 1));
            ctx->iter_eager_done = true;
            ran = true;
        } else {
            cudaGraph_t g;
            // no other thread may allocate (and so synchronise the device)
            // while this stream is being captured
            std::lock_guard<std::recursive_mutex> lk(device_mutex());
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            set_capturing(true);
            int rc = 0;
            // the cut copies are compacted (and the tree refit) once, at the
            // iteration's last step
            for (int i = 0; i < PRUNE_STEPS && !rc; ++i)
                rc = ctx->enqueue_step(fStep, false, bNoCut != 0, i, G, i == PRUNE_STEPS - 1);
            const int bound = ctx->slot_bound(G);
            if (!rc && mover_prune(ctx->M, ctx->L, ctx->mkey_lo, ctx->mkey_inv, fCvg, ctx->ss, st, bound,
                                   ctx->opt_curve & 1))
                rc = SKID_ECUDA;
            set_capturing(false);
            cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (rc) return ctx->fail(rc);
            if (ce) return ctx->fail_cuda(ce);
            size_t nn = 0;
            cudaGraphGetNodes(g, nullptr, &nn);
            std::vector<cudaGraphNode_t> nodes(nn);
            if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
            ctx->iter_graph_kernels[gs] = 0;
            for (auto nd : nodes) {
                cudaGraphNodeType ty;
                if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                    ++ctx->iter_graph_kernels[gs];
            }
            ce = cudaGraphInstantiate(&ctx->iter_graph[gs], g, 0);
            cudaGraphDestroy(g);
            if (ce) return ctx->fail_cuda(ce);
            ctx->g_fStep[gs] = fStep;
            ctx->g_fCvg[gs] = fCvg;
            ctx->g_nocut[gs] = bNoCut != 0;
            ctx->g_stats[gs] = ctx->field_stats_on;
            ctx->g_bound[gs] = bound;
            ctx->g_key[gs] = ctx->graph_key();
        }
    }
    if (!ran) {
        CK(cudaGraphLaunch(ctx->iter_graph[gs], st));
        note_launch((int)ctx->iter_graph_kernels[gs]);
    }
    int vals[2];
    CK(cudaMemcpyAsync(&vals[0], ctx->M.d_nA, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&vals[1], ctx->C.d_n2, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (int rc = ctx->sync_check()) return rc;
    ctx->collect_field_times(PRUNE_STEPS);
    ctx->tim.moving_ms += ctx->timer_stop();
    ctx->nActive = vals[0];
    if (nActive) *nActive = vals[0];
    if (nScatter) *nScatter = vals[1];
    return 0;
}

int skid_reactivate_move(skid_ctx *ctx)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_MOVE) return ctx->fail(SKID_ESTATE);
    iota_kernel<<<grid_for(ctx->nMove), 256, 0, ctx->st>>>(ctx->M.act.p, ctx->nMove); skid::note_launch();
    CK(cudaMemcpyAsync(ctx->M.d_nA, &ctx->nMove, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
    ctx->nActive = ctx->nMove;
    return ctx->sync_check();
}

int skid_get_moved(skid_ctx *ctx, float *pos)
{
    if (!ctx || !pos) return SKID_EINVAL;
    if (ctx->stage < STAGE_LOADED) return ctx->fail(SKID_ESTATE);
    int n = ctx->n;
    float *d = ctx->raw.p;
    pos4_to_xyz<<<grid_for(n), 256, 0, ctx->st>>>(ctx->pos4.p, n, d); skid::note_launch();
    if (ctx->stage >= STAGE_MOVE && ctx->nMove > 0)
        moved_to_iorder<<<grid_for(ctx->nMove), 256, 0, ctx->st>>>(ctx->M.mpos.p, ctx->M.mio.p,
                                                                   ctx->nMove, d); skid::note_launch();
    CK(cudaMemcpyAsync(pos, d, 3 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
    return ctx->sync_check();
}

int skid_get_timings(skid_ctx *ctx, skid_timings *t)
{
    if (!ctx || !t) return SKID_EINVAL;
    *t = ctx->tim;
    double fb[2] = {0.0, 0.0};
    if (cudaMemcpyAsync(fb, ctx->d_fbytes, sizeof(fb), cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess ||
        cudaStreamSynchronize(ctx->st) != cudaSuccess)
        return ctx->fail(SKID_ECUDA);
    t->gather_launches = (long long)fb[1];
    t->kernel_launches = launches_total();
    t->field_bytes = fb[0];
    return 0;
}

int skid_field_stats(skid_ctx *ctx, int enable, unsigned long long *out4)
{
    if (!ctx) return SKID_EINVAL;
    if (!ctx->d_fstats) {
        std::lock_guard<std::recursive_mutex> lk(device_mutex());
        if (cudaMalloc((void **)&ctx->d_fstats, 4 * sizeof(unsigned long long))) ctx->d_fstats = nullptr;
    }
    if (!ctx->d_fstats)
        return ctx->fail(SKID_ENOMEM);
    if (out4) {
        CK(cudaMemcpyAsync(out4, ctx->d_fstats, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    CK(cudaMemsetAsync(ctx->d_fstats, 0, 4 * sizeof(unsigned long long), ctx->st));
    ctx->field_stats_on = enable != 0;   // graphs are recaptured on the next iteration
    return 0;
}

int skid_set_option(skid_ctx *ctx, const char *name, double value)
{
    if (!ctx || !name) return SKID_EINVAL;
    int v = (int)value;
    if (!strcmp(name, "field_movers_per_warp")) {
        if (v != 0 && v != 1 && v != 4 && v != 8 && v != 16 && v != 32 && v != 64) return SKID_EINVAL;
        ctx->opt_G = v;
    } else if (!strcmp(name, "field_g64_min")) {
        if (v < 0) return SKID_EINVAL;
        ctx->opt_g64_min = v;
    } else if (!strcmp(name, "field_g32_min")) {
        if (v < 0) return SKID_EINVAL;
        ctx->opt_g32_min = v;
    } else if (!strcmp(name, "field_g16_min")) {
        if (v < 0) return SKID_EINVAL;
        ctx->opt_g16_min = v;
    } else if (!strcmp(name, "field_g8_min")) {
        if (v < 0) return SKID_EINVAL;
        ctx->opt_g8_min = v;
    } else if (!strcmp(name, "field_g4_min")) {
        if (v < 0) return SKID_EINVAL;
        ctx->opt_g4_min = v;
    } else if (!strcmp(name, "unbind_warp_max")) {
        if (v != -1 && v != 0 && v != 32 && v != 64 && v != 128 && v != 256 && v != 512 && v != 1024)
            return SKID_EINVAL;
        ctx->opt_unbind_tw = v;
    } else if (!strcmp(name, "unbind_block")) {
        if (v != -1 && v != 128 && v != 256 && v != 512 && v != 1024) return SKID_EINVAL;
        ctx->opt_unbind_bs = v;
    } else if (!strcmp(name, "unbind_per_group")) {
        ctx->opt_unbind_per_group = v != 0;
    } else if (!strcmp(name, "unbind_cluster_min")) {
        if (v != -1 && v != 0 && v < 1024) return SKID_EINVAL;
        ctx->opt_unbind_clu_min = v;
    } else if (!strcmp(name, "curve")) {
        if (v < 0 || v > 7) return SKID_EINVAL;
        ctx->opt_curve = v;
        ctx->drop_graphs();   // the captured prunes and re-sorts carry the curve
    } else if (!strcmp(name, "field_unfused")) {
        ctx->opt_field_unfused = v != 0;
        ctx->drop_graphs();
    } else if (!strcmp(name, "unbind_retune")) {
        ctx->U.tuned_tw = ctx->U.tuned_bs = ctx->U.tuned_cs = -1;
        ctx->U.ntune = 0;
    } else {
        return SKID_EINVAL;
    }
    return 0;
}

int skid_get_option(skid_ctx *ctx, const char *name, double *value)
{
    if (!ctx || !name || !value) return SKID_EINVAL;
    if (!strcmp(name, "field_movers_per_warp")) *value = ctx->opt_G;
    else if (!strcmp(name, "field_g32_min")) *value = ctx->opt_g32_min;
    else if (!strcmp(name, "field_g64_min")) *value = ctx->opt_g64_min;
    else if (!strcmp(name, "field_g16_min")) *value = ctx->opt_g16_min;
    else if (!strcmp(name, "field_g8_min")) *value = ctx->opt_g8_min;
    else if (!strcmp(name, "field_g4_min")) *value = ctx->opt_g4_min;
    else if (!strcmp(name, "unbind_warp_max")) *value = ctx->U.used_tw;
    else if (!strcmp(name, "unbind_block")) *value = ctx->U.used_bs;
    else if (!strcmp(name, "unbind_per_group")) *value = ctx->opt_unbind_per_group;
    else if (!strcmp(name, "unbind_cluster_min")) *value = ctx->opt_unbind_clu_min;
    else if (!strcmp(name, "curve")) *value = ctx->opt_curve;
    else if (!strcmp(name, "unbind_cluster_size")) *value = ctx->U.used_cs;
    else if (!strcmp(name, "unbind_cluster_groups")) *value = ctx->U.used_nclu;
    else if (!strcmp(name, "unbind_tune_candidates")) *value = ctx->U.ntune;
    else if (!strcmp(name, "unbind_pot_ms")) *value = ctx->U.pot_ms;
    else if (!strcmp(name, "unbind_remove_ms")) *value = ctx->U.remove_ms;
    else if (!strncmp(name, "unbind_tune_ms", 14)) {
        int k = atoi(name + 14);
        if (k < 0 || k >= 32 || k >= ctx->U.ntune) return SKID_EINVAL;
        *value = ctx->U.tune_ms[k];
    }
    else if (!strcmp(name, "field_unfused")) *value = ctx->opt_field_unfused;
    else return SKID_EINVAL;
    return 0;
}

int skid_stream(skid_ctx *ctx, void **stream)
{
    if (!ctx || !stream) return SKID_EINVAL;
    *stream = (void *)ctx->st;
    return 0;
}

int skid_knn_ball2(skid_ctx *ctx, int n, const float *pos, int k, float *ball2)
{
    if (!ctx || n < 0 || !pos || !ball2 || k < 1 || k > n) return SKID_EINVAL;
    cudaStream_t st = ctx->st;
    Tree &t = ctx->probe_tree;
    DBuf<float> &xyz = ctx->probe_f;
    DBuf<float4> &p4 = ctx->probe_p4;
    if (dalloc(xyz, 3 * (size_t)n + n) || dalloc(p4, n)) return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(xyz.p, pos, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
    xyz_to_pos4<<<grid_for(n), 256, 0, st>>>(xyz.p, n, p4.p); skid::note_launch();
    CK(tree_build(t, p4.p, n, false, ctx->ss, st));
    float *b_sorted = xyz.p;   // reuse: sorted results, then unsorted
    float *b_out = xyz.p + n;
    CK(knn_ball2(t, k, ctx->L, ctx->per, b_sorted, ctx->d_scal + SC_WORK, ctx->knn_heap, st));
    unsort_floats<<<grid_for(n), 256, 0, st>>>(t.perm.p, b_sorted, n, b_out); skid::note_launch();
    CK(cudaMemcpyAsync(ball2, b_out, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    return ctx->sync_check();
}

int skid_field(skid_ctx *ctx, int nm, const float *mpos, float *acc)
{
    if (!ctx || nm < 0 || !mpos || !acc) return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    if (int rc = field_probe(ctx, nm, mpos)) return rc;
    CK(cudaMemcpyAsync(acc, ctx->probe_acc.p, 3 * (size_t)nm * sizeof(float), cudaMemcpyDeviceToHost,
                       ctx->st));
    return ctx->sync_check();
}

int skid_field_adjoint(skid_ctx *ctx, int nm, const float *mpos, const float *w, float *dLdy)
{
    if (!ctx || nm < 0 || !mpos || !w || !dLdy) return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    if (int rc = field_probe(ctx, nm, mpos)) return rc;
    cudaStream_t st = ctx->st;
    if (dalloc(ctx->adj.win, nm > 0 ? nm : 1)) return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(ctx->adj.win.p, w, (size_t)nm * sizeof(float), cudaMemcpyHostToDevice, st));
    scale_field<<<grid_for(nm), 256, 0, st>>>(ctx->probe_acc.p, ctx->adj.win.p, nm); skid::note_launch();
    CK(cudaMemcpyAsync(dLdy, ctx->probe_acc.p, 3 * (size_t)nm * sizeof(float), cudaMemcpyDeviceToHost, st));
    return ctx->sync_check();
}

int skid_density_adjoint(skid_ctx *ctx, const float *w, float *dLdx, int mode)
{
    if (!ctx || !w || !dLdx ||
        (mode != SKID_ADJ_RECOMPUTE && mode != SKID_ADJ_STORED && mode != SKID_ADJ_AUTO))
        return SKID_EINVAL;
    if (ctx->stage < STAGE_DENSITY) return ctx->fail(SKID_ESTATE);
    if (ctx->par.nSmooth < 2) return ctx->fail(SKID_EINVAL);
    cudaStream_t st = ctx->st;
    int n = ctx->n;
    if (dalloc(ctx->adj.win, n > 0 ? n : 1)) return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(ctx->adj.win.p, w, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
    cudaError_t e = density_adjoint(ctx->stree, ctx->sb2.p, ctx->sidx.p, ctx->adj.win.p, n, ctx->L,
                                    ctx->per, mode, ctx->par.nSmooth, ctx->adj, ctx->d_scal + SC_WORK,
                                    ctx->d_status, st);
    if (e == cudaErrorMemoryAllocation) return ctx->fail(SKID_ENOMEM);
    CK(e);
    CK(cudaMemcpyAsync(dLdx, ctx->adj.out.p, 3 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
    return ctx->sync_check();
}

}  // extern "C"
