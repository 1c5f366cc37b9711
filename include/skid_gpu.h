/*
 * skid_gpu.h -- C ABI of libskidgpu, the GB300 (sm_103a) implementation of
 * SKID's group-finding path (N-BodyShop/skid v1.4.1).
 *
 * The reference has no plugin or FFI layer: its driver main.c calls the
 * internal API of kd.h:338-365 and smooth1.h:94-99 in a fixed order
 * (main.c:347-485).  Each entry point below replaces one of those calls (or
 * one step of main.c) and says which.  A host program (the `skid` CLI in
 * skid_gb300/host, or Python through ctypes) makes the same sequence of calls
 * and writes the same output files.
 *
 * Conventions
 *  - Every call returns 0 on success or a negative SKID_E* code; nothing in
 *    the library exits, asserts or prints (progress lines are the caller's).
 *  - A context owns all device memory; host buffers are the caller's and are
 *    copied (per-particle arrays are indexed by iOrder: gas, dark, star).
 *  - Device-side failures (a bounded wait that ran out, a capacity overflow)
 *    are latched in a device status word and returned by the next call that
 *    synchronises; skid_last_error() repeats the first one.
 *  - One context per host thread; calls on a context are serialised on its
 *    own CUDA stream.  Contexts are independent.
 *  - Positions are float32; FP64 appears only in per-group sums.
 */
#ifndef SKID_GPU_H
#define SKID_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKID_OK 0
#define SKID_EINVAL -1      /* bad argument or call order                   */
#define SKID_ENOMEM -2      /* device or host allocation failed             */
#define SKID_ECUDA -3       /* CUDA runtime error                           */
#define SKID_ETIMEOUT -4    /* a bounded device-side wait ran out           */
#define SKID_EOVERFLOW -5   /* an internal capacity was exceeded            */
#define SKID_ENODEV -6      /* no usable sm_103 device                      */
#define SKID_ESTATE -7      /* call made in the wrong pipeline state        */
#define SKID_ETOOLARGE -8   /* request exceeds a fixed (static) capacity     */

#define SKID_SOFT_PLUMMER 1 /* kd.h:24 */
#define SKID_SOFT_SPLINE 2  /* kd.h:25 */

typedef struct skid_ctx skid_ctx;

/* Box and smoothing parameters fixed for a context (kdInit, kd.c:46-82,
 * and smInit, smooth1.c:8-29).  period[] is FLT_MAX when not periodic. */
typedef struct skid_params {
    float period[3];
    float center[3];
    int periodic;        /* -p given: periodic replica scatterers (main.c:279) */
    int nSmooth;         /* -s (main.c:185-190) */
    int device;          /* CUDA device ordinal */
} skid_params;

/* One group as written to .gtp / .stat (PGROUP, kd.h:45-55). */
typedef struct skid_group {
    int nMembers;
    float fMass;
    float rel[3];
    float rCenter[3];
    float rBound[3];
    float vcm[3];
    float fRadius;
} skid_group;

/* Device time per stage, milliseconds (CUDA events); the reference prints
 * user CPU time per stage (main.c:486-494). */
typedef struct skid_timings {
    float density_ms, moving_ms, fof_ms, micro_ms, groups_ms, unbind_ms, toosmall_ms;
    long long gather_launches;  /* move-field kernel launches so far */
    long long kernel_launches;  /* all kernels launched so far, all contexts */
    double field_ms;            /* summed CUDA-event time of the move-field kernel */
    double field_bytes;         /* its algorithmic bytes: 24 per active mover
                                   (position read + write) + 20 per live
                                   scatterer (position, mass, fBall2) */
} skid_timings;

/* kdInit (kd.c:46-82) + smInit (smooth1.c:8-29).  nSmooth >= 1 and every
 * period > 0 (FLT_MAX: no period), else SKID_EINVAL before any device work. */
int skid_create(skid_ctx **pctx, const skid_params *par);

/* kdFinish (kd.c:1842-1850) + smFinish (smooth1.c:32-38). */
int skid_destroy(skid_ctx *ctx);

/* Error text for a SKID_E* code. */
const char *skid_strerror(int code);

/* First error latched on this context (0 if none). */
int skid_last_error(const skid_ctx *ctx);

/* Text of the first CUDA runtime error behind a SKID_ECUDA ("none" if none). */
const char *skid_last_cuda_error(const skid_ctx *ctx);

/* kdReadTipsy (kd.c:122-222), data part: copies particles to the device.
 * pos/vel are float[3n], mass/soft/temp float[n]; temp may be NULL (0).
 * soft is hsmooth for gas and eps for dark and star.  n = nGas + nDark +
 * nStar must be 1 .. 2^28 with no negative count (else SKID_EINVAL). */
int skid_set_particles(skid_ctx *ctx, int nGas, int nDark, int nStar, double time,
                       const float *pos, const float *vel, const float *mass,
                       const float *soft, const float *temp);

/* Return to the state right after skid_set_particles, keeping the particles
 * on the device (for repeated runs on one snapshot; no reference
 * counterpart: the reference reads its input once). */
int skid_restart(skid_ctx *ctx);

/* The snapshot straight from its TIPSY particle records (kdReadTipsy,
 * kd.c:122-222): `records` holds the nGas gas (12 words), nDark dark (9)
 * and nStar star (11) records that follow the header, in file order, XDR
 * big-endian when bStandard.  One copy to the device and a kernel unpacks
 * them (pinned host memory from skid_host_alloc makes the copy a single
 * DMA).  bytes must equal the records' size exactly. */
int skid_set_tipsy(skid_ctx *ctx, int nGas, int nDark, int nStar, double time, int bStandard,
                   const void *records, size_t bytes);

/* Page-locked host memory for input buffers (no context needed); returns
 * SKID_ENOMEM where it cannot be had (no device), *ptr = NULL. */
int skid_host_alloc(size_t bytes, void **ptr);
int skid_host_free(void *ptr);

/* kdScatterActive (kd.c:669-693) with ScatterCriterion (kd.c:600-627). */
int skid_scatter_active(skid_ctx *ctx, int bGasAndDark, int bGasOnly, int *nScatter);

/* kdBuildTree (kd.c:371-460) + smDensityInit (smooth1.c:132-335): kNN ball
 * radii, symmetric SPH density, periodic replica scatterers. */
int skid_density(skid_ctx *ctx, int *nExtraScat);

/* kdOutDensity's data (kd.c:1526-1547): density and fBall2 by iOrder
 * (0 and -1 for particles that are not scatterers).  Either may be NULL. */
int skid_get_density(skid_ctx *ctx, float *rho, float *ball2);

/* kdInitMove (kd.c:630-666) with CutCriterion (kd.c:555-597). */
int skid_init_move(skid_ctx *ctx, float fDensMin, float fTempMax, float fMassMax,
                   int bGasAndDark, int bGasOnly, int *nMove);

/* smAccDensity (smooth1.c:408-518) followed by kdMoveParticles
 * (kd.c:702-732): one move step of the active movers.  bInitial selects the
 * first-step cut (main.c:396-401); bNoCut is the -nsp switch.  nScatter gets
 * the live scatterer copies after the cut. */
int skid_move_step(skid_ctx *ctx, float fStep, int bInitial, int bNoCut, int *nScatter);

/* kdPruneInactive (kd.c:735-793). */
int skid_prune_inactive(skid_ctx *ctx, float fCvg, int *nActive);

/* One outer iteration of main.c:409-419 (PRUNE_STEPS move steps and a
 * prune), replayed from a CUDA graph after its first capture. */
int skid_move_iterate(skid_ctx *ctx, float fStep, float fCvg, int bNoCut,
                      int *nActive, int *nScatter);

/* kdReactivateMove (kd.c:796-799). */
int skid_reactivate_move(skid_ctx *ctx);

/* kdFoF (kd.c:802-917): friends-of-friends over all movers at link length
 * fTau.  nGroup gets the number of groups (group 0 excluded).  Groups are
 * numbered by ascending smallest member iOrder. */
int skid_fof(skid_ctx *ctx, float fTau, int *nGroup);

/* kdInitpGroup (kd.c:969-1005) + kdCalcCenter (kd.c:1013-1075). */
int skid_group_centers(skid_ctx *ctx);

/* kdInGroup (kd.c:920-962) + kdInitpGroup + kdReadCenter (kd.c:1083-1196):
 * unbind-only mode.  grp[n] holds group ids by iOrder; centers (nGroup
 * records, index 0 unused) gives rCenter and vcm, or NULL to use the centre
 * of mass. */
int skid_set_groups(skid_ctx *ctx, const int *grp, int nGroup, const skid_group *centers);

/* kdSetSoft (kd.c:103-110). */
int skid_set_soft(skid_ctx *ctx, float fEps);

/* kdUnbind (kd.c:1299-1466) with kdCellPot/kdSubPot/kdAddScoopPot
 * (grav.c:8-135).  a = 1/(1+z); aH = a*H(a) (kd.c:1317-1318).  Every group
 * runs in one launch.  nUnbound gets the particles removed. */
int skid_unbind(skid_ctx *ctx, int iSoftType, float fScoop, int bGasAndDark, int bNoUnbind,
                int nMaxMembers, float G, float z, float a, float aH, int *nUnbound);

/* kdTooSmall (kd.c:1251-1293). */
int skid_too_small(skid_ctx *ctx, int nMembers, int *nGroup);

/* Group ids by iOrder (kdOutGroup, kd.c:1502-1523) and the group records
 * (kdWriteGroup, kd.c:1611-1687; fRadius computed here).  groups has room
 * for nGroup+1 records (index 0 = ungrouped).  Either may be NULL. */
int skid_get_groups(skid_ctx *ctx, int *grp, skid_group *groups);

/* Per-group columns 2-12 of the .stat table (kdOutStats, kd.c:1703-1839),
 * computed on the device after skid_too_small with the reference's own
 * float and FP64 roundings.  The reference prints sqrt of the three
 * fVcirc2 values and of fROuter2 (kd.c:1819-1833); columns 13-21 are the
 * records' rCenter, vcm and rBound. */
typedef struct skid_stat {
    int nMembers;
    float fTotMass, fGasMass, fStarMass;
    float fVcirc2Max;    /* G M(<r)/r at its maximum outside 2 eps (fVcirc)     */
    float fVcirc2Half;   /* G M/r where the enclosed mass first exceeds half    */
    float fVcirc2Outer;  /* G M/r at the outermost member (flVcirc)              */
    float fRVmax, fRHalf;
    float fROuter2;      /* squared radius of the outermost member              */
    float fVdisp;        /* 1-D velocity dispersion, Hubble flow included       */
} skid_stat;

/* kdOutStats' per-group statistics for groups 1..nGroup (stats[0] unused;
 * stats holds nGroup+1 records).  G, fExp = 1/(1+z) and fExpHub = a H(a) as
 * for skid_unbind; fDensMin and fTempMax select the gas mass that counts.
 * Replaces kd.c:1703-1839 (the file writing stays with the caller). */
int skid_group_stats(skid_ctx *ctx, float G, float fExp, float fExpHub, float fDensMin,
                     float fTempMax, skid_stat *stats);

/* Moved positions by iOrder (kdOutVector's data, kd.c:1550-1608); input
 * position for particles that never moved. */
int skid_get_moved(skid_ctx *ctx, float *pos);

/* Densities after the first-step cut set untouched scatterers to 0
 * (smooth1.c:463-470); kdOutStats reads these (kd.c:1790). */
int skid_get_final_density(skid_ctx *ctx, float *rho);

/* The stage times and the move-field figures of the current run (they
 * restart with skid_set_particles, skid_set_tipsy and skid_restart);
 * kernel_launches counts from process start. */
int skid_get_timings(skid_ctx *ctx, skid_timings *t);

/* Work counters of the move-field kernel (no reference counterpart): with
 * enable set, later move steps count tree nodes visited, leaves visited,
 * candidate scatterer tests and in-ball hits.  out4 (may be NULL) receives
 * the counts so far; the counters then restart from zero. */
int skid_field_stats(skid_ctx *ctx, int enable, unsigned long long *out4);

/* Tuning knobs (no reference counterpart).  Names:
 *   "field_movers_per_warp"  0 = by active count (default), or 64 (two per
 *                            lane), 32, 16, 8, 4, 1
 *   "field_g64_min"          active movers at or above which 64 per warp
 *                            (default 0: never)
 *   "field_g32_min"          active movers at or above which 32 per warp
 *   "field_g16_min"          ... 16 per warp
 *   "field_g8_min"           ... 8 per warp
 *   "field_g4_min"           ... 4 per warp (one per warp below)
 *   "unbind_warp_max"        groups up to this size get one warp each in the
 *                            removal loop: 0, 32, 64, 128, 256, 512, 1024,
 *                            or -1 = autotuned
 *                            (default: every candidate is timed on the first
 *                            skid_unbind of the context, the fastest is kept)
 *   "unbind_block"           threads per block for larger groups: 128, 256,
 *                            512, 1024, or -1 = autotuned
 *   "unbind_cluster_min"     groups above this size (at least 1024) may be
 *                            removed by a cluster of blocks that hold their
 *                            members in shared memory; 0 = never; -1 (the
 *                            default) = above 2048, and only when the
 *                            autotuner measured that faster
 *   "unbind_per_group"       1: one potential and one removal launch per group
 *                            (the reference's serial loop, for comparison)
 *   "unbind_retune"          forget the autotuned schedule
 *   "field_unfused"          1: every move step runs the field as a separate
 *                            gradient pass (field to memory, then a move
 *                            kernel) instead of the fused adjoint-and-move
 *                            kernel (for comparison; set before
 *                            skid_init_move)
 * Returns SKID_EINVAL for an unknown name or value. */
int skid_set_option(skid_ctx *ctx, const char *name, double value);

/* Current value of a knob; for "unbind_warp_max" and "unbind_block" the
 * schedule the last skid_unbind used, "unbind_cluster_size" and
 * "unbind_cluster_groups" its cluster size (1: none) and the number of groups
 * it removed on clusters, "unbind_tune_candidates" the number of
 * schedules the autotuner timed, "unbind_tune_ms<k>" the removal time of
 * candidate k (warp sizes outer, block sizes inner), "unbind_pot_ms" and
 * "unbind_remove_ms" the potential and removal times of the last
 * skid_unbind (CUDA events). */
int skid_get_option(skid_ctx *ctx, const char *name, double *value);

/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order their own work against the library's (no reference counterpart). */
int skid_stream(skid_ctx *ctx, void **stream);

/* ---- Batched volumes (no reference counterpart: the reference runs one
 * snapshot per process). ---- */

/* One independent volume of a batch: inputs as for skid_set_particles and
 * skid_params, per-volume nSmooth and link length; outputs filled in. */
typedef struct skid_volume {
    int nGas, nDark, nStar;
    double time;
    const float *pos, *vel, *mass, *soft, *temp;   /* host, by iOrder; temp may be NULL */
    float period[3], center[3];
    int periodic;
    int nSmooth;
    float fTau, fCvg, fScoop;    /* fCvg, fScoop <= 0: tau/2 and 2 tau (main.c:337-342) */
    int *grp;                    /* out: n final group ids, or NULL */
    skid_group *groups;          /* out: groups_cap records (index 0 = ungrouped), or NULL */
    int groups_cap;
    int nGroup, nGroupFoF, nUnbound, nIter;   /* out */
    float device_ms;             /* out: summed stage time of this volume */
    int status;                  /* out: 0, or the SKID_E* code that stopped it */
    char message[96];            /* out: the CUDA error text behind a SKID_ECUDA */
} skid_volume;

/* Flags shared by every volume of a batch (main.c:82-345 meanings). */
typedef struct skid_batch_flags {
    float fDensMin, fTempMax, fMassMax;
    int nMembers, nMaxMembers;
    int bGasAndDark, bGasOnly, bForceInitialCut, bNoUnbind, bNoCut;
    int iSoftType, bEps;
    float fEps;
    float G, z, a, aH;           /* a = 1/(1+z), aH = a*H(a) (kd.c:1317-1318) */
    int maxIter;                 /* 0: until every mover has converged */
} skid_batch_flags;

/* Run the whole pipeline on nVol independent volumes of uneven sizes on one
 * GPU.  nWorkers host workers (each with its own context and CUDA stream)
 * take volumes largest first from a shared queue, so the pipelines of many
 * volumes run on the GPU at once; each worker's context reuses its device
 * memory across volumes (its move-iteration graphs are captured again for
 * every volume, whose period and step length they carry), and every volume
 * takes the usual fixed removal schedule rather than tuning one.
 * Results per volume are those of the single-volume sequence.  Returns 0 if
 * every volume succeeded, else the first failing volume's status; a volume
 * with a period that is not positive or nSmooth below 1 makes the call
 * return SKID_EINVAL before any work. */
int skid_batch_run(skid_volume *vols, int nVol, const skid_batch_flags *flags, int nWorkers,
                   int device);

/* ---- Adjoints (no reference counterpart). ---- */

#define SKID_ADJ_RECOMPUTE 0   /* find the neighbour pairs by walking the tree again */
#define SKID_ADJ_STORED 1      /* gather every ball's members once and reuse the lists */
#define SKID_ADJ_AUTO 2        /* stored while the lists fit in a quarter of the free
                                  device memory, else recomputed */

/* Gradient of L = sum_i w_i rho_i (rho the symmetric SPH density of
 * skid_density, smooth1.c:132-276) with respect to the scatterer positions,
 * the neighbour sets of skid_density held fixed: pair terms in both balls
 * that hold a pair, plus each smoothing length's dependence on its k-th
 * neighbour (h_i = |x_i - x_K(i)|/2).  w[n] by iOrder (non-scatterers'
 * entries unused); dLdx[3n] by iOrder (0 for non-scatterers).  FP32
 * arithmetic and accumulation.  SKID_ADJ_STORED keeps n_scatter*(nSmooth+16)
 * indices on the device until the next skid_density; SKID_ADJ_RECOMPUTE
 * stores nothing.  Needs nSmooth >= 2.  Call after skid_density (any later
 * stage). */
int skid_density_adjoint(skid_ctx *ctx, const float *w, float *dLdx, int mode);

/* Query-position adjoint of the density field of the live scatterer copies,
 * rho_f(y) = sum_c m_c W(|y - x_c|, h_c): dLdy[3i] = w[i] grad rho_f(y_i)
 * for nm points y (mpos[3nm]).  The move field of smAccDensity
 * (smooth1.c:436-508) is -grad rho_f: the move kernel is this adjoint with a
 * unit cotangent, fused with the step. */
int skid_field_adjoint(skid_ctx *ctx, int nm, const float *mpos, const float *w, float *dLdy);

/* Potential energy of groups and its gradient.  For the nSel groups sel[]
 * (ids of the grouping made by skid_group_centers or skid_set_groups; call
 * before skid_unbind), E[s] = -1/2 sum_{i != j in g} G m_i m_j
 * psi(r_ij, eps_i + eps_j) with kdCellPot's pair potential (grav.c:8-36,
 * grav.h:11-31) on coordinates relative to the group's reference point
 * (kd.c:1338-1352); FP32 pair sums, FP64 group totals.  With dLdx non-NULL,
 * dLdx[3n] (by iOrder) receives sum_s v[s] dE[s]/dx (0 outside the selected
 * groups). */
int skid_potential_adjoint(skid_ctx *ctx, int iSoftType, float G, int nSel, const int *sel,
                           const float *v, double *E, float *dLdx);

/* ---- Allocation-free entry point. ---- */

/* Limits of skid_knn_ball2_noalloc's static scratch. */
#define SKID_NOALLOC_MAX_POINTS 65536
#define SKID_NOALLOC_MAX_K 256

/* k-th nearest-neighbour squared distance (self included) of each of n
 * points among the same points, like skid_knn_ball2, for callers that cannot
 * allocate device memory (a framework that owns the device allocator; a loop
 * that cannot afford cudaMalloc's implicit synchronisation).  No reference
 * counterpart.  d_pos (float[3n]) and d_ball2 (float[n]) are DEVICE pointers
 * owned by the caller; period[3] is host memory (FLT_MAX: not periodic);
 * stream is a cudaStream_t (NULL: the default stream) and the call returns
 * once the work is queued on it.  Every intermediate lives in one
 * file-scope device array of about 5 MB that each GPU loading the library
 * keeps until exit; nothing is allocated or freed.  n above
 * SKID_NOALLOC_MAX_POINTS or k above SKID_NOALLOC_MAX_K returns
 * SKID_ETOOLARGE.  The first call on a device looks up the array's address
 * there (make it before any stream capture).  Calls share the array: calls
 * whose work overlaps on the GPU race. */
int skid_knn_ball2_noalloc(const float *d_pos, int n, int k, const float period[3],
                           float *d_ball2, void *stream);

/* ---- Stage probes with explicit inputs (parity tests, adjoint checks). ---- */

/* k-th nearest neighbour squared distance (self included) of each of n
 * points among the same points (smooth1.c:41-243), written to ball2. */
int skid_knn_ball2(skid_ctx *ctx, int n, const float *pos, int k, float *ball2);

/* The move field at nm positions from the context's current live scatterer
 * copies (smooth1.c:436-508): acc[3*nm] = sum m/(pi h^5) F(q) (x_c - y). */
int skid_field(skid_ctx *ctx, int nm, const float *mpos, float *acc);

/* Friends-of-friends of n explicit points (kd.c:802-917). */
int skid_fof_points(skid_ctx *ctx, int n, const float *pos, float fTau, int *grp, int *nGroup);

/* The float pair factor of the unbinding potentials ("dir" of kdCellPot,
 * kdSubPot and kdAddScoopPot, grav.c:25-30,50-55,118-124, with SPLINE_POT of
 * grav.h:11-31) for n pairs of squared distance d2[i] and summed softening
 * twoh[i] (host arrays), computed on the device into out[n]:
 *   SKID_PAIR_USED       the form the unbinding kernels use;
 *   SKID_PAIR_FP64       the reference's FP64 expression, rounded to float;
 *   SKID_PAIR_SPLINE_FF  the float-float spline alone, NaN where it leaves
 *                        the value to the FP64 expression.
 * A numerics check: the first two must agree bit for bit. */
#define SKID_PAIR_USED 0
#define SKID_PAIR_FP64 1
#define SKID_PAIR_SPLINE_FF 2
int skid_pair_factor(int n, const float *d2, const float *twoh, int plummer, int mode, float *out);

#ifdef __cplusplus
}
#endif
#endif
