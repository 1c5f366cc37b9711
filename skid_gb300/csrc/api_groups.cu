// C ABI, group stages: friends-of-friends, group centres, unbind-only input,
// unbinding, too-small removal and the output records (main.c:424-485).
#include <cfloat>
#include <cstring>
#include <vector>

#include "ctx.h"

using namespace skid;

namespace {

__global__ void reorder_movers(const uint32_t *__restrict__ perm, int n, const float4 *__restrict__ o,
                               const int *__restrict__ io, float4 *__restrict__ o2,
                               int *__restrict__ io2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t j = perm[i];
        o2[i] = o[j];
        io2[i] = io[j];
    }
}

__global__ void xyz_to_p4(const float *__restrict__ xyz, int n, float4 *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = make_float4(xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2],
                             0.0f);
}

__global__ void iota_k(int *p, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

__global__ void scatter_movers(const float4 *__restrict__ mpos, const int *__restrict__ mio, int nm,
                               float4 *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x)
        out[mio[i]] = mpos[i];
}

__global__ void set_centres(const skid_group *__restrict__ in, int ng, skid_group *__restrict__ rec)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x + 1; g < ng; g += gridDim.x * blockDim.x) {
        for (int d = 0; d < 3; ++d) {
            rec[g].rCenter[d] = in[g].rCenter[d];
            rec[g].vcm[d] = in[g].vcm[d];
        }
    }
}

__global__ void set_soft_k(float4 *vel4, int n, float eps, float *keep)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (keep) keep[i] = vel4[i].w;
        vel4[i].w = eps;
    }
}

__global__ void gather_group0(const int *__restrict__ members, const int *__restrict__ start,
                              const int *__restrict__ count, const float4 *__restrict__ pos4,
                              float4 *__restrict__ out)
{
    int s = start[0], c = count[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c; i += gridDim.x * blockDim.x)
        out[i] = pos4[members[s + i]];
}

__global__ void gather_usoft(const uint32_t *__restrict__ perm, const int *__restrict__ members,
                             const int *__restrict__ start, int n0, const float4 *__restrict__ vel4,
                             float *__restrict__ out)
{
    int s = start[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n0; i += gridDim.x * blockDim.x)
        out[i] = vel4[members[s + perm[i]]].w;
}

}  // namespace

extern "C" {

int skid_fof(skid_ctx *ctx, float fTau, int *nGroup)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_MOVE) return ctx->fail(SKID_ESTATE);
    cudaStream_t st = ctx->st;
    ctx->timer_start();
    int nm = ctx->nMove;
    CK(cudaMemsetAsync(ctx->grp.p, 0, ctx->n * sizeof(int), st));
    // kdFoF (kd.c:814) makes every mover active again
    CK(fof_run(ctx->mtree, ctx->M.mpos.p, nm, ctx->M.mio.p, ctx->n, fTau, ctx->L, ctx->per, ctx->ss,
               ctx->parent, ctx->fof_minio, ctx->fof_flag, ctx->grp.p, ctx->d_scal + SC_NG,
               ctx->d_scal + SC_WORK, ctx->d_status, st));
    if (nm > 0) {
        // keep movers in Hilbert order of their current positions (coherent
        // warps for the micro-steps)
        if (dalloc(ctx->moved4, ctx->n)) return ctx->fail(SKID_ENOMEM);
        reorder_movers<<<grid_for(nm), 256, 0, st>>>(ctx->mtree.perm.p, nm, ctx->M.mold.p,
                                                     ctx->M.mio.p, ctx->moved4.p, ctx->M.act2.p); skid::note_launch();
        // mtree.pos holds the positions in the new order
        CK(cudaMemcpyAsync(ctx->M.mpos.p, ctx->mtree.pos.p, nm * sizeof(float4),
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(ctx->M.mold.p, ctx->moved4.p, nm * sizeof(float4),
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(ctx->M.mio.p, ctx->M.act2.p, nm * sizeof(int), cudaMemcpyDeviceToDevice,
                           st));
        iota_k<<<grid_for(nm), 256, 0, st>>>(ctx->M.act.p, nm); skid::note_launch();
        CK(cudaMemcpyAsync(ctx->M.d_nA, &ctx->nMove, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    int ng = 0;
    if (int rc = ctx->read_int(ctx->d_scal + SC_NG, &ng)) return rc;
    ctx->G.nGroup = ng + 1;
    ctx->nActive = nm;
    ctx->tim.fof_ms += ctx->timer_stop();

    if (nGroup) *nGroup = ng;
    ctx->stage = STAGE_FOF;
    return 0;
}

int skid_group_centers(skid_ctx *ctx)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_FOF) return ctx->fail(SKID_ESTATE);
    cudaStream_t st = ctx->st;
    ctx->timer_start();
    int n = ctx->n;
    if (dalloc(ctx->moved4, n)) return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(ctx->moved4.p, ctx->pos4.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    if (ctx->nMove > 0)
        scatter_movers<<<grid_for(ctx->nMove), 256, 0, st>>>(ctx->M.mpos.p, ctx->M.mio.p, ctx->nMove,
                                                             ctx->moved4.p); skid::note_launch();
    CK(group_order(ctx->grp.p, n, ctx->G.nGroup, ctx->ss, ctx->G, st));
    CK(group_props(ctx->G, ctx->pos4.p, ctx->vel4.p, ctx->moved4.p, ctx->L, ctx->wrap_hi(),
                   ctx->wrap_lo(), false, false, st));
    if (int rc = ctx->sync_check()) return rc;
    ctx->tim.groups_ms += ctx->timer_stop();

    ctx->stage = STAGE_GROUPS;
    return 0;
}

int skid_set_groups(skid_ctx *ctx, const int *grp, int nGroup, const skid_group *centers)
{
    if (!ctx || !grp || nGroup < 1) return SKID_EINVAL;
    if (ctx->stage < STAGE_LOADED) return ctx->fail(SKID_ESTATE);
    int n = ctx->n;
    for (int i = 0; i < n; ++i)
        if (grp[i] < 0 || grp[i] >= nGroup) return ctx->fail(SKID_EINVAL);
    cudaStream_t st = ctx->st;
    CK(cudaMemcpyAsync(ctx->grp.p, grp, n * sizeof(int), cudaMemcpyHostToDevice, st));
    ctx->G.nGroup = nGroup;
    CK(group_order(ctx->grp.p, n, nGroup, ctx->ss, ctx->G, st));
    CK(group_props(ctx->G, ctx->pos4.p, ctx->vel4.p, ctx->pos4.p, ctx->L, ctx->wrap_hi(),
                   ctx->wrap_lo(), centers == nullptr, true, st));
    if (centers) {
        DBuf<skid_group> &tmp = ctx->G.rec2;
        if (dalloc(tmp, nGroup)) return ctx->fail(SKID_ENOMEM);
        CK(cudaMemcpyAsync(tmp.p, centers, nGroup * sizeof(skid_group), cudaMemcpyHostToDevice, st));
        set_centres<<<grid_for(nGroup), 256, 0, st>>>(tmp.p, nGroup, ctx->G.rec.p); skid::note_launch();
    }
    if (int rc = ctx->sync_check()) return rc;
    ctx->stage = STAGE_GROUPS;
    return 0;
}

int skid_potential_adjoint(skid_ctx *ctx, int iSoftType, float G, int nSel, const int *sel,
                           const float *v, double *E, float *dLdx)
{
    if (!ctx || nSel < 0 || (nSel > 0 && (!sel || !E)) || (dLdx && !v)) return SKID_EINVAL;
    if (iSoftType != SKID_SOFT_PLUMMER && iSoftType != SKID_SOFT_SPLINE) return SKID_EINVAL;
    if (ctx->stage != STAGE_GROUPS) return ctx->fail(SKID_ESTATE);
    for (int s = 0; s < nSel; ++s)
        if (sel[s] < 1 || sel[s] >= ctx->G.nGroup) return ctx->fail(SKID_EINVAL);
    cudaStream_t st = ctx->st;
    cudaError_t e = potential_adjoint(ctx->G, ctx->pos4.p, ctx->vel4.p, ctx->n, ctx->L, G,
                                      iSoftType == SKID_SOFT_PLUMMER, nSel, sel, v, dLdx != nullptr,
                                      ctx->adj, st);
    if (e == cudaErrorMemoryAllocation) return ctx->fail(SKID_ENOMEM);
    CK(e);
    if (nSel) CK(cudaMemcpyAsync(E, ctx->adj.E.p, nSel * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (dLdx)
        CK(cudaMemcpyAsync(dLdx, ctx->adj.out.p, 3 * (size_t)ctx->n * sizeof(float), cudaMemcpyDeviceToHost,
                           st));
    return ctx->sync_check();
}

int skid_set_soft(skid_ctx *ctx, float fEps)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_LOADED) return ctx->fail(SKID_ESTATE);
    float *keep = nullptr;
    if (!ctx->soft_changed) {
        if (dalloc(ctx->soft_orig, ctx->n > 0 ? ctx->n : 1)) return ctx->fail(SKID_ENOMEM);
        keep = ctx->soft_orig.p;
        ctx->soft_changed = true;
    }
    set_soft_k<<<grid_for(ctx->n), 256, 0, ctx->st>>>(ctx->vel4.p, ctx->n, fEps, keep); skid::note_launch();
    ctx->soft_min = fEps;
    return ctx->sync_check();
}

int skid_unbind(skid_ctx *ctx, int iSoftType, float fScoop, int bGasAndDark, int bNoUnbind,
                int nMaxMembers, float G, float z, float a, float aH, int *nUnbound)
{
    (void)bGasAndDark;   // the scoop term is applied for every input (kd.c:1379-1384)
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_GROUPS) return ctx->fail(SKID_ESTATE);
    cudaStream_t st = ctx->st;
    ctx->timer_start();
    // tree over the ungrouped particles for the scoop (kd.c:1324-1325)
    int n0 = 0;
    CK(cudaMemcpyAsync(&n0, ctx->G.count.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    DBuf<float4> &u4 = ctx->probe_p4;
    if (dalloc(u4, n0 > 0 ? n0 : 1) || dalloc(ctx->U.usoft, n0 > 0 ? n0 : 1)) return ctx->fail(SKID_ENOMEM);
    if (n0 > 0) {
        gather_group0<<<grid_for(n0), 256, 0, st>>>(ctx->G.members.p, ctx->G.start.p, ctx->G.count.p,
                                                    ctx->pos4.p, u4.p); skid::note_launch();
    }
    CK(tree_build(ctx->utree, u4.p, n0, false, ctx->ss, st));
    if (n0 > 0)
        gather_usoft<<<grid_for(n0), 256, 0, st>>>(ctx->utree.perm.p, ctx->G.members.p, ctx->G.start.p,
                                                   n0, ctx->vel4.p, ctx->U.usoft.p); skid::note_launch();
    UnbindParams P;
    P.period = ctx->L;
    P.per = ctx->per;
    P.fScoop = fScoop;
    P.nmax = nMaxMembers;
    P.G = G;
    P.a = a;
    P.aH = aH;
    P.opz = (float)(1.0 + (double)z);
    P.z = z;
    P.plummer = iSoftType == SKID_SOFT_PLUMMER;
    P.subpot = ctx->inType == 1 || ctx->inType == 4;   // kd.c:1441
    P.nounbind = bNoUnbind != 0;
    if (ctx->ensure_mass_soft()) return ctx->fail(SKID_ECUDA);
    P.scale = ctx->pot_scale(G);
    P.n = ctx->n;
    P.tw = ctx->opt_unbind_tw;
    P.bs = ctx->opt_unbind_bs;
    P.clu_auto = ctx->opt_unbind_clu_min < 0;
    P.clu_min = P.clu_auto ? 2048 : ctx->opt_unbind_clu_min;
    P.per_group = ctx->opt_unbind_per_group;
    CK(unbind_run(ctx->G, ctx->G.gof.p, ctx->n, ctx->pos4.p, ctx->vel4.p, ctx->utree, P, ctx->grp.p,
                  ctx->d_scal + SC_NUNB, ctx->ss, ctx->U, st));
    int nu = 0;
    if (int rc = ctx->read_int(ctx->d_scal + SC_NUNB, &nu)) return rc;
    ctx->tim.unbind_ms += ctx->timer_stop();

    if (nUnbound) *nUnbound = nu;
    ctx->stage = STAGE_UNBOUND;
    return 0;
}

int skid_too_small(skid_ctx *ctx, int nMembers, int *nGroup)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_GROUPS) return ctx->fail(SKID_ESTATE);
    ctx->timer_start();
    CK(too_small(ctx->G, ctx->grp.p, ctx->n, nMembers, ctx->d_scal + SC_NG2, ctx->ss, ctx->st));
    int ng = 0;
    if (int rc = ctx->read_int(ctx->d_scal + SC_NG2, &ng)) return rc;
    ctx->G.nGroup = ng + 1;
    CK(group_radius(ctx->G, ctx->grp.p, ctx->n, ctx->pos4.p, ctx->L, ctx->st));
    if (int rc = ctx->sync_check()) return rc;
    ctx->tim.toosmall_ms += ctx->timer_stop();

    if (nGroup) *nGroup = ng;
    ctx->stage = STAGE_FINAL;
    return 0;
}

int skid_get_groups(skid_ctx *ctx, int *grp, skid_group *groups)
{
    if (!ctx) return SKID_EINVAL;
    if (ctx->stage < STAGE_FOF) return ctx->fail(SKID_ESTATE);
    if (grp) CK(cudaMemcpyAsync(grp, ctx->grp.p, ctx->n * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    if (groups) {
        if (ctx->stage < STAGE_GROUPS) return ctx->fail(SKID_ESTATE);
        if (ctx->stage < STAGE_FINAL)
            CK(group_radius(ctx->G, ctx->grp.p, ctx->n, ctx->pos4.p, ctx->L, ctx->st));
        CK(cudaMemcpyAsync(groups, ctx->G.rec.p, ctx->G.nGroup * sizeof(skid_group),
                           cudaMemcpyDeviceToHost, ctx->st));
    }
    return ctx->sync_check();
}

int skid_fof_points(skid_ctx *ctx, int n, const float *pos, float fTau, int *grp, int *nGroup)
{
    if (!ctx || n < 0 || !pos || !grp) return SKID_EINVAL;
    cudaStream_t st = ctx->st;
    DBuf<float> &xyz = ctx->probe_f;
    DBuf<float4> &p4 = ctx->probe_p4;
    DBuf<int> &io = ctx->probe_i;
    DBuf<int> &g = ctx->probe_i2;
    if (dalloc(xyz, 3 * (size_t)n) || dalloc(p4, n) || dalloc(io, n) || dalloc(g, n))
        return ctx->fail(SKID_ENOMEM);
    CK(cudaMemcpyAsync(xyz.p, pos, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
    xyz_to_p4<<<grid_for(n), 256, 0, st>>>(xyz.p, n, p4.p); skid::note_launch();
    iota_k<<<grid_for(n), 256, 0, st>>>(io.p, n); skid::note_launch();
    CK(fof_run(ctx->probe_tree, p4.p, n, io.p, n, fTau, ctx->L, ctx->per, ctx->ss, ctx->parent,
               ctx->fof_minio, ctx->fof_flag, g.p, ctx->d_scal + SC_NG, ctx->d_scal + SC_WORK,
               ctx->d_status, st));
    CK(cudaMemcpyAsync(grp, g.p, n * sizeof(int), cudaMemcpyDeviceToHost, st));
    int ng = 0;
    if (int rc = ctx->read_int(ctx->d_scal + SC_NG, &ng)) return rc;
    if (nGroup) *nGroup = ng;
    return 0;
}

}  // extern "C"
