// skid_batch_run: many independent volumes on one GPU.
//
// A volume's pipeline alternates kernels with small host decisions (counts
// read back to size the next stage, the outer move loop's stopping test), so
// one volume alone leaves most of the GPU idle when it is small.  The batch
// runs the pipelines of several volumes at once: each host worker owns a
// context (its own stream and device memory) and takes volumes from a shared
// queue, largest first, so the long volumes start early and the short ones
// fill the gaps.  Contexts keep their buffers from one volume to the next,
// and use the usual removal schedule rather than tuning their own.  The calls
// per volume are exactly the single-volume sequence of the reference driver
// (main.c:374-485), so every volume's result equals a run of its own.
#include <algorithm>
#include <cstdio>
#include <atomic>
#include <cfloat>
#include <thread>
#include <vector>

#include "ctx.h"

using namespace skid;

namespace {

constexpr int BATCH_PRUNE_STEPS = 5;     // main.c:13
constexpr double BATCH_MICRO_STEP = 0.1; // main.c:14

// Point an existing context at another volume's box and smoothing count.
void reconfigure(skid_ctx *ctx, const skid_volume &v)
{
    for (int d = 0; d < 3; ++d) {
        ctx->par.period[d] = v.period[d];
        ctx->par.center[d] = v.center[d];
    }
    ctx->par.periodic = v.periodic;
    ctx->par.nSmooth = v.nSmooth;
    ctx->L = make_float3(v.period[0], v.period[1], v.period[2]);
    ctx->hL = make_float3(0.5f * v.period[0], 0.5f * v.period[1], 0.5f * v.period[2]);
    ctx->per = v.period[0] < 0.25f * FLT_MAX;
    ctx->drop_graphs();
}

int run_volume(skid_ctx *ctx, skid_volume &v, const skid_batch_flags &f)
{
    reconfigure(ctx, v);
    v.nGroup = v.nGroupFoF = v.nUnbound = v.nIter = 0;
    v.device_ms = 0.0f;
    int rc;
    if ((rc = skid_set_particles(ctx, v.nGas, v.nDark, v.nStar, v.time, v.pos, v.vel, v.mass, v.soft,
                                 v.temp)))
        return rc;
    const float tau = v.fTau;
    const float cvg = v.fCvg > 0.0f ? v.fCvg : (float)(0.5 * tau);
    const float scoop = v.fScoop > 0.0f ? v.fScoop : (float)(2.0 * tau);
    const float step = (float)(0.5 * cvg);
    int ns = 0, nx = 0, nm = 0, nsc = 0;
    if ((rc = skid_scatter_active(ctx, f.bGasAndDark, f.bGasOnly, &ns))) return rc;
    if ((rc = skid_density(ctx, &nx))) return rc;
    if ((rc = skid_init_move(ctx, f.fDensMin, f.fTempMax, f.fMassMax, f.bGasAndDark, f.bGasOnly, &nm)))
        return rc;
    int inType = (v.nDark ? 1 : 0) | (v.nGas ? 2 : 0) | (v.nStar ? 4 : 0);
    int initial = inType == 1 || f.bForceInitialCut;   // bAllowInitialCut, kd.c:696-699
    if ((rc = skid_move_step(ctx, step, initial, f.bNoCut, &nsc))) return rc;
    int na = nm, it = 1;
    while (na) {
        if (f.maxIter > 0 && it > f.maxIter) break;
        if ((rc = skid_move_iterate(ctx, step, cvg, f.bNoCut, &na, &nsc))) return rc;
        ++it;
    }
    v.nIter = it - 1;
    int ng = 0;
    if ((rc = skid_fof(ctx, tau, &ng))) return rc;
    v.nGroupFoF = ng;
    if ((rc = skid_reactivate_move(ctx))) return rc;
    float micro = (float)(BATCH_MICRO_STEP * step);
    for (int i = 0; i < BATCH_PRUNE_STEPS; ++i)
        if ((rc = skid_move_step(ctx, micro, 0, f.bNoCut, &nsc))) return rc;
    if ((rc = skid_group_centers(ctx))) return rc;
    if (f.bEps && (rc = skid_set_soft(ctx, f.fEps))) return rc;
    int nu = 0;
    if ((rc = skid_unbind(ctx, f.iSoftType, scoop, f.bGasAndDark, f.bNoUnbind, f.nMaxMembers, f.G, f.z,
                          f.a, f.aH, &nu)))
        return rc;
    v.nUnbound = nu;
    if ((rc = skid_too_small(ctx, f.nMembers, &ng))) return rc;
    v.nGroup = ng;
    bool fits = v.groups && v.groups_cap >= ng + 1;
    if ((rc = skid_get_groups(ctx, v.grp, fits ? v.groups : nullptr))) return rc;
    skid_timings t;
    if ((rc = skid_get_timings(ctx, &t))) return rc;
    v.device_ms = t.density_ms + t.moving_ms + t.fof_ms + t.micro_ms + t.groups_ms + t.unbind_ms +
                  t.toosmall_ms;
    if (v.groups && !fits) return SKID_EOVERFLOW;
    return 0;
}

}  // namespace

extern "C" int skid_batch_run(skid_volume *vols, int nVol, const skid_batch_flags *flags, int nWorkers,
                              int device)
{
    if (nVol < 0 || (nVol > 0 && !vols) || !flags || nWorkers < 1) return SKID_EINVAL;
    if (nVol == 0) return 0;
    for (int i = 0; i < nVol; ++i) {
        vols[i].status = SKID_ENODEV;   // until a worker runs it
        vols[i].message[0] = 0;
        for (int d = 0; d < 3; ++d)
            if (!(vols[i].period[d] > 0.0f) || vols[i].nSmooth < 1) return SKID_EINVAL;
    }
    // largest volumes first
    std::vector<int> order(nVol);
    for (int i = 0; i < nVol; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        long long na = (long long)vols[a].nGas + vols[a].nDark + vols[a].nStar;
        long long nb = (long long)vols[b].nGas + vols[b].nDark + vols[b].nStar;
        return na > nb;
    });
    if (nWorkers > nVol) nWorkers = nVol;
    std::atomic<int> next(0);
    std::vector<int> wrc(nWorkers, 0);
    auto worker = [&](int w) {
        skid_params par{};
        const skid_volume &v0 = vols[order[0]];
        for (int d = 0; d < 3; ++d) {
            par.period[d] = v0.period[d];
            par.center[d] = v0.center[d];
        }
        par.periodic = v0.periodic;
        par.nSmooth = v0.nSmooth > 0 ? v0.nSmooth : 1;
        par.device = device;
        skid_ctx *ctx = nullptr;
        int rc = skid_create(&ctx, &par);
        if (rc) {
            wrc[w] = rc;
            // no context: the volumes this worker would have taken are left to the others
            return;
        }
        // Each worker's context would otherwise time the 18 candidate removal
        // schedules on its first volume, every batch: the volumes take the
        // schedule the tuner picks on clustered snapshots instead (a warp per
        // group of up to 1024 members, 512-thread blocks above).
        skid_set_option(ctx, "unbind_warp_max", 1024);
        skid_set_option(ctx, "unbind_block", 512);
        for (;;) {
            int k = next.fetch_add(1);
            if (k >= nVol) break;
            skid_volume &v = vols[order[k]];
            v.status = run_volume(ctx, v, *flags);
            snprintf(v.message, sizeof(v.message), "%s",
                     v.status == SKID_ECUDA ? skid_last_cuda_error(ctx) : "");
        }
        skid_destroy(ctx);
    };
    std::vector<std::thread> th;
    for (int w = 0; w < nWorkers; ++w) th.emplace_back(worker, w);
    for (auto &t : th) t.join();
    bool any_ctx = false;
    for (int w = 0; w < nWorkers; ++w) any_ctx = any_ctx || wrc[w] == 0;
    if (!any_ctx) return wrc[0];
    for (int i = 0; i < nVol; ++i)
        if (vols[i].status) return vols[i].status;
    return 0;
}
