/*
 * skid -- command-line driver over libskidgpu.
 *
 * Same flags, defaults, stdin input, progress lines and output files as the
 * reference driver (main.c:17-495): reads a TIPSY snapshot from standard
 * input, runs density -> move -> FoF -> micro-steps -> centres -> unbind ->
 * too-small through the C ABI in skid_gpu.h, and writes <name>.grp and
 * <name>.gtp, plus .den (-den), .ray (-ray) and .stat (-stats).  Two flags
 * are new: -nsp keeps every scatterer (no scatterer cut) and -maxiter caps
 * the outer move iterations.  The closing table reports device time per
 * stage from CUDA events instead of the reference's user CPU time.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "skid_gpu.h"
#include "tipsy_io.h"

#define PRUNE_STEPS 5     /* main.c:13 */
#define MICRO_STEP 0.1    /* main.c:14 */
#define T_DARK 1
#define T_GAS 2
#define T_STAR 4

typedef struct options {
    float fTau, z, Omega0, Lambda, fQuintess, G, H0;
    int nSmooth;
    float fDensMin, fTempMax, fMassMax, fCvg, fScoop, fStep;
    int nMembers, nMaxMembers;
    int bNoUnbind, bGasAndDark, bGasOnly, bUnbindOnly, bForceInitialCut;
    int bPeriodic, iSoftType, bEps;
    float fEps;
    float period[3], center[3];
    char achGroup[256], achName[256];
    int bOutRay, bOutDens, bOutStats, bOutDiag, bStandard, bNoScatterCut, maxIter;
} options;

static void usage(void)
{
    fprintf(stderr,
            "USAGE:\n"
            "skid -tau <fLinkLength> [OPTIONAL ARGUMENTS]\n"
            "     reads TIPSY BINARY input file from stdin\n"
            "     [-std]\n"
            "COSMOLOGY and UNITS arguments:\n"
            "     [-z <fRedShift>] [-O <fOmega>]\n"
            "     [-G <fGravConst>] [-H <fHubble>]\n"
            "     [-Lambda <fLambda>] [-Q <fQuintessense]\n"
            "GROUP FINDING arguments:\n"
            "     [-s <nSmooth>] [-d <fMinDensity>] [-t <fMaxTemp>]\n"
            "     [-cvg <fConvergeRadius>] [-scoop <fScoopRadius>]\n"
            "     [-m <nMinMembers>] [-nu] [-gd] [-unbind <GroupName>[.grp]]\n"
            "     [-M <fMaxMass>] [-fic] [-go] [-maxgroup nMaxMembers]\n"
            "     [-nsp] [-maxiter <nIterations>]\n"
            "GRAVITATIONAL SOFTENING arguments:\n"
            "     [-spline] [-plummer] [-e <fSoft>]\n"
            "PERIODIC BOX specification:\n"
            "     [-p <xyzPeriod>]\n"
            "     [-c <xyzCenter>]\n"
            "     [-cx <xCenter>] [-cy <yCenter>] [-cz <zCenter>]\n"
            "OUTPUT arguments:\n"
            "     [-o <Output Name>] [-ray] [-den] [-stats] [-diag]\n");
    exit(1);
}

/* Option parsing with the reference's defaults and derived values
 * (main.c:82-345). */
static void parse(int argc, char **argv, options *o)
{
    memset(o, 0, sizeof(*o));
    o->Omega0 = 1.0f;
    o->G = 1.0f;
    o->nSmooth = 64;
    o->fTempMax = FLT_MAX;
    o->fMassMax = FLT_MAX;
    o->nMembers = 8;
    o->nMaxMembers = INT_MAX;
    o->iSoftType = SKID_SOFT_SPLINE;
    for (int d = 0; d < 3; ++d) o->period[d] = FLT_MAX;
    strcpy(o->achName, "skid");
    int bTau = 0, bCvg = 0, bScoop = 0;
    int i = 1;
#define NEXT() (++i < argc ? argv[i++] : (usage(), (char *)0))
    while (i < argc) {
        const char *a = argv[i];
        if (!strcmp(a, "-tau")) { o->fTau = (float)atof(NEXT()); bTau = 1; }
        else if (!strcmp(a, "-z")) o->z = (float)atof(NEXT());
        else if (!strcmp(a, "-O")) o->Omega0 = (float)atof(NEXT());
        else if (!strcmp(a, "-Lambda")) o->Lambda = (float)atof(NEXT());
        else if (!strcmp(a, "-Q")) o->fQuintess = (float)atof(NEXT());
        else if (!strcmp(a, "-G")) o->G = (float)atof(NEXT());
        else if (!strcmp(a, "-H")) o->H0 = (float)atof(NEXT());
        else if (!strcmp(a, "-s")) o->nSmooth = atoi(NEXT());
        else if (!strcmp(a, "-d")) o->fDensMin = (float)atof(NEXT());
        else if (!strcmp(a, "-t")) o->fTempMax = (float)atof(NEXT());
        else if (!strcmp(a, "-M")) o->fMassMax = (float)atof(NEXT());
        else if (!strcmp(a, "-fic")) { o->bForceInitialCut = 1; ++i; }
        else if (!strcmp(a, "-cvg")) { o->fCvg = (float)atof(NEXT()); bCvg = 1; }
        else if (!strcmp(a, "-scoop")) { o->fScoop = (float)atof(NEXT()); bScoop = 1; }
        else if (!strcmp(a, "-m")) o->nMembers = atoi(NEXT());
        else if (!strcmp(a, "-maxgroup")) o->nMaxMembers = atoi(NEXT());
        else if (!strcmp(a, "-nu")) { o->bNoUnbind = 1; ++i; }
        else if (!strcmp(a, "-gd")) { o->bGasAndDark = 1; ++i; }
        else if (!strcmp(a, "-go")) { o->bGasOnly = 1; ++i; }
        else if (!strcmp(a, "-unbind")) {
            snprintf(o->achGroup, sizeof(o->achGroup), "%s", NEXT());
            o->bUnbindOnly = 1;
        }
        else if (!strcmp(a, "-spline")) { o->iSoftType = SKID_SOFT_SPLINE; ++i; }
        else if (!strcmp(a, "-plummer")) { o->iSoftType = SKID_SOFT_PLUMMER; ++i; }
        else if (!strcmp(a, "-e")) { o->fEps = (float)atof(NEXT()); o->bEps = 1; }
        else if (!strcmp(a, "-p")) {
            float v = (float)atof(NEXT());
            o->period[0] = o->period[1] = o->period[2] = v;
            o->bPeriodic = 1;
        }
        else if (!strcmp(a, "-c")) {
            float v = (float)atof(NEXT());
            o->center[0] = o->center[1] = o->center[2] = v;
        }
        else if (!strcmp(a, "-cx")) o->center[0] = (float)atof(NEXT());
        else if (!strcmp(a, "-cy")) o->center[1] = (float)atof(NEXT());
        else if (!strcmp(a, "-cz")) o->center[2] = (float)atof(NEXT());
        else if (!strcmp(a, "-o")) snprintf(o->achName, sizeof(o->achName), "%s", NEXT());
        else if (!strcmp(a, "-ray")) { o->bOutRay = 1; ++i; }
        else if (!strcmp(a, "-den")) { o->bOutDens = 1; ++i; }
        else if (!strcmp(a, "-stats")) { o->bOutStats = 1; ++i; }
        else if (!strcmp(a, "-diag")) { o->bOutDiag = 1; ++i; }
        else if (!strcmp(a, "-std")) { o->bStandard = 1; ++i; }
        else if (!strcmp(a, "-nsp")) { o->bNoScatterCut = 1; ++i; }
        else if (!strcmp(a, "-maxiter")) o->maxIter = atoi(NEXT());
        else usage();
    }
#undef NEXT
    if (!bTau) usage();
    if (!bCvg) o->fCvg = (float)(0.5 * o->fTau);
    if (!bScoop) o->fScoop = (float)(2.0 * o->fTau);
    o->fStep = (float)(0.5 * o->fCvg);
}

/* a = 1/(1+z) and a*H(a) as floats (kd.c:1317-1318; H(a) of cosmo.c:46-58
 * with no radiation term). */
static void expansion(const options *o, float *a, float *aH)
{
    float fa = (float)(1.0 / (1.0 + o->z));
    double da = fa;
    double curv = 1.0 - (double)o->Omega0 - (double)o->Lambda - (double)o->fQuintess;
    double h = (double)o->H0 *
               sqrt((double)o->Omega0 * da + curv * da * da +
                    (double)o->fQuintess * da * da * sqrt(da) + (double)o->Lambda * da * da * da * da) /
               (da * da);
    *a = fa;
    *aH = (float)(da * h);
}

static skid_ctx *g_ctx;

static void die_on(int rc, const char *what)
{
    if (rc == SKID_OK) return;
    fprintf(stderr, "skid: %s failed: %s", what, skid_strerror(rc));
    if (rc == SKID_ECUDA && g_ctx) fprintf(stderr, " (%s)", skid_last_cuda_error(g_ctx));
    fprintf(stderr, "\n");
    exit(2);
}

/* ---- .stat: per-group statistics (kdOutStats, kd.c:1703-1839) ----
 * The statistics are computed on the device (skid_group_stats); the host
 * prints them in the reference's format, with sqrt of the squared columns
 * taken in double as the reference's printf arguments are. */

static int write_stats(const char *path, const options *o, skid_ctx *ctx, const skid_group *gr,
                       int nGroup)
{
    float fExp, fExpHub;
    expansion(o, &fExp, &fExpHub);
    skid_stat *st = malloc(((size_t)nGroup + 1) * sizeof(skid_stat));
    if (!st) return -1;
    die_on(skid_group_stats(ctx, o->G, fExp, fExpHub, o->fDensMin, o->fTempMax, st),
           "skid_group_stats");
    FILE *fp = fopen(path, "w");
    if (!fp) {
        free(st);
        return -1;
    }
    for (int g = 1; g <= nGroup; ++g) {
        const skid_stat *q = &st[g];
        const skid_group *G = &gr[g];
        if (q->nMembers <= 0) continue;
        fprintf(fp, "%d %d %g %g %g %g %g %g %g %g %g %g %g %g %g %g %g %g %g %g %g\n", g,
                q->nMembers, q->fTotMass, q->fGasMass, q->fStarMass, sqrt(q->fVcirc2Max),
                sqrt(q->fVcirc2Half), sqrt(q->fVcirc2Outer), q->fRVmax, q->fRHalf,
                sqrt(q->fROuter2), q->fVdisp, G->rCenter[0], G->rCenter[1], G->rCenter[2],
                G->vcm[0], G->vcm[1], G->vcm[2], G->rBound[0], G->rBound[1], G->rBound[2]);
    }
    free(st);
    return fclose(fp) ? -1 : 0;
}

/* ---- unbind-only inputs: kdInGroup (kd.c:920-962), kdReadCenter (kd.c:1083-1196) ---- */

static int read_unbind_inputs(const options *o, const snapshot *s, int **grp, int *nGroup,
                              skid_group **centers)
{
    char base[300], path[320], err[512];
    snprintf(base, sizeof(base), "%s", o->achGroup);
    size_t L = strlen(base);
    if (L >= 4 && !strcmp(base + L - 4, ".grp")) base[L - 4] = 0;
    snprintf(path, sizeof(path), "%s.grp", base);
    int n = read_grp(path, grp, err, sizeof(err));
    if (n < 0) {
        fprintf(stderr, "%s\n", err);
        return -1;
    }
    if (n != s->n) {
        fprintf(stderr, "ERROR: Mismatched number of particles: %d in %s, %d in the TIPSY input\n",
                n, path, s->n);
        return -1;
    }
    int ng = 0;
    for (int i = 0; i < n; ++i) ng = (*grp)[i] > ng ? (*grp)[i] : ng;
    *nGroup = ng;
    *centers = NULL;
    snprintf(path, sizeof(path), "%s.gtp", base);
    int ns = 0;
    float *mass = NULL, *pos = NULL, *vel = NULL;
    int rc = tipsy_read_gtp(path, o->bStandard, &ns, &mass, &pos, &vel, err, sizeof(err));
    if (rc < 0) {
        fprintf(stderr, "%s\n", err);
        return -1;
    }
    if (rc == 1) {
        if (ns != ng) {
            fprintf(stderr, "ERROR: grp and gtp files don't match: %d vs. %d.\n", ns, ng);
            return -1;
        }
        *centers = calloc((size_t)ng + 1, sizeof(skid_group));
        for (int g = 1; g <= ng; ++g)
            for (int d = 0; d < 3; ++d) {
                (*centers)[g].rCenter[d] = pos[3 * (size_t)(g - 1) + d];
                (*centers)[g].vcm[d] = vel[3 * (size_t)(g - 1) + d];
            }
    }
    free(mass);
    free(pos);
    free(vel);
    return 0;
}

/* Wall-clock phases of the process, printed to stderr when SKID_WALL_TIMES
 * is set (1: the phases as they run; 2: also a CUDA start-up probe before
 * the input is read, which separates driver start-up from reading). */
static double wall_ms(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return 1e3 * (double)t.tv_sec + 1e-6 * (double)t.tv_nsec;
}

static int g_wall = 0;
static double g_wall_t = 0.0;

static void wall_mark(const char *phase)
{
    if (!g_wall) return;
    const double t = wall_ms();
    fprintf(stderr, "wall_ms %s %.3f\n", phase, t - g_wall_t);
    g_wall_t = t;
}

int main(int argc, char **argv)
{
    options o;
    {
        const char *w = getenv("SKID_WALL_TIMES");
        g_wall = w ? atoi(w) : 0;
        g_wall_t = wall_ms();
        if (g_wall) fprintf(stderr, "wall_abs_ms main %.3f\n", g_wall_t);
    }
    parse(argc, argv, &o);
    if (g_wall >= 2) {
        void *probe = NULL;
        if (skid_host_alloc(16, &probe) == SKID_OK) skid_host_free(probe);
        wall_mark("cuda_start");
    }
    printf("SKID v1.4.1 (GB300)\n");
    /* the particle records as they lie in the file, in page-locked memory;
     * they are unpacked on the device (skid_set_tipsy) */
    tipsy_raw raw;
    char err[512];
    if (tipsy_read_raw(stdin, o.bStandard, &raw, err, sizeof(err))) {
        fprintf(stderr, "skid: %s\n", err);
        return 2;
    }
    snapshot s;
    memset(&s, 0, sizeof(s));
    s.time = raw.time;
    s.nGas = raw.nGas;
    s.nDark = raw.nDark;
    s.nStar = raw.nStar;
    s.n = raw.n;
    printf("nDark:%d nGas:%d nStar:%d\n", s.nDark, s.nGas, s.nStar);
    fflush(stdout);
    wall_mark("read");

    skid_params par;
    memset(&par, 0, sizeof(par));
    for (int d = 0; d < 3; ++d) {
        par.period[d] = o.period[d];
        par.center[d] = o.center[d];
    }
    par.periodic = o.bPeriodic;
    par.nSmooth = o.nSmooth;
    par.device = 0;
    die_on(skid_create(&g_ctx, &par), "skid_create");
    skid_ctx *ctx = g_ctx;
    wall_mark("create");
    /* One run per process: timing the 18 candidate removal schedules would
     * cost more than it saves, so the tool takes the schedule the tuner
     * picks on clustered snapshots (a warp per group of up to 1024 members,
     * 512-thread blocks above); SKID_UNBIND_TUNE=1 tunes instead. */
    {
        const char *tune = getenv("SKID_UNBIND_TUNE");
        if (!tune || strcmp(tune, "1") != 0) {
            die_on(skid_set_option(ctx, "unbind_warp_max", 1024), "skid_set_option");
            die_on(skid_set_option(ctx, "unbind_block", 512), "skid_set_option");
        }
    }
    die_on(skid_set_tipsy(ctx, raw.nGas, raw.nDark, raw.nStar, raw.time, o.bStandard, raw.records,
                          raw.bytes),
           "skid_set_tipsy");
    if (o.bOutRay) {   /* the initial positions, for the displacements */
        s.pos = malloc(3 * (size_t)(s.n > 0 ? s.n : 1) * sizeof(float));
        tipsy_raw_positions(&raw, o.bStandard, s.pos);
    }
    tipsy_raw_free(&raw);
    wall_mark("upload");

    int nFoF = 0;
    int inType = (s.nDark ? T_DARK : 0) | (s.nGas ? T_GAS : 0) | (s.nStar ? T_STAR : 0);
    float *moved = NULL;
    if (o.bUnbindOnly) {
        int *grp_in = NULL;
        skid_group *centers = NULL;
        if (read_unbind_inputs(&o, &s, &grp_in, &nFoF, &centers)) return 1;
        die_on(skid_set_groups(ctx, grp_in, nFoF + 1, centers), "skid_set_groups");
        free(grp_in);
        free(centers);
    } else {
        int nScat = 0, nExtra = 0, nActive = 0;
        die_on(skid_scatter_active(ctx, o.bGasAndDark, o.bGasOnly, &nScat), "skid_scatter_active");
        die_on(skid_density(ctx, &nExtra), "skid_density");
        if (o.bPeriodic) printf("nExtraScat:%d\n", nExtra);
        if (o.bOutDens) {
            float *rho = malloc((size_t)(s.n > 0 ? s.n : 1) * sizeof(float));
            char path[300];
            die_on(skid_get_density(ctx, rho, NULL), "skid_get_density");
            snprintf(path, sizeof(path), "%s.den", o.achName);
            if (write_den(path, s.n, rho)) fprintf(stderr, "skid: cannot write %s\n", path);
            free(rho);
        }
        die_on(skid_init_move(ctx, o.fDensMin, o.fTempMax, o.fMassMax, o.bGasAndDark, o.bGasOnly,
                              &nActive),
               "skid_init_move");
        int initial = inType == T_DARK || o.bForceInitialCut;   /* bAllowInitialCut, kd.c:113-119 */
        die_on(skid_move_step(ctx, o.fStep, initial, o.bNoScatterCut, &nScat), "skid_move_step");
        printf("Ittr:%d nActive:%d nScatter:%d\n", 0, nActive, nScat);
        fflush(stdout);
        for (int it = 1; nActive; ++it) {
            if (o.maxIter && it > o.maxIter) break;
            die_on(skid_move_iterate(ctx, o.fStep, o.fCvg, o.bNoScatterCut, &nActive, &nScat),
                   "skid_move_iterate");
            printf("Ittr:%d nActive:%d nScatter:%d\n", it, nActive, nScat);
            fflush(stdout);
        }
        die_on(skid_fof(ctx, o.fTau, &nFoF), "skid_fof");
        die_on(skid_reactivate_move(ctx), "skid_reactivate_move");
        float micro = (float)(MICRO_STEP * o.fStep);
        for (int i = 0; i < PRUNE_STEPS; ++i) {
            die_on(skid_move_step(ctx, micro, 0, o.bNoScatterCut, &nScat), "skid_move_step");
            printf("Microstep:%d nScatter:%d\n", i + 1, nScat);
            fflush(stdout);
        }
        if (o.bOutRay) {
            moved = malloc(3 * (size_t)(s.n > 0 ? s.n : 1) * sizeof(float));
            die_on(skid_get_moved(ctx, moved), "skid_get_moved");
        }
        die_on(skid_group_centers(ctx), "skid_group_centers");
    }
    if (o.bEps) die_on(skid_set_soft(ctx, o.fEps), "skid_set_soft");
    printf("Groups before Unbind:%d\n", nFoF);
    fflush(stdout);
    float a, aH;
    expansion(&o, &a, &aH);
    int nUnbound = 0, nGroup = 0;
    die_on(skid_unbind(ctx, o.iSoftType, o.fScoop, o.bGasAndDark, o.bNoUnbind, o.nMaxMembers, o.G,
                       o.z, a, aH, &nUnbound),
           "skid_unbind");
    printf("Number of particles Unbound:%d\n", nUnbound);
    die_on(skid_too_small(ctx, o.nMembers, &nGroup), "skid_too_small");
    printf("Number of Groups:%d\n", nGroup);
    fflush(stdout);
    wall_mark("pipeline");

    int *grp = malloc((size_t)(s.n > 0 ? s.n : 1) * sizeof(int));
    skid_group *gr = malloc(((size_t)nGroup + 1) * sizeof(skid_group));
    die_on(skid_get_groups(ctx, grp, gr), "skid_get_groups");
    wall_mark("fetch");
    char path[300];
    snprintf(path, sizeof(path), "%s.grp", o.achName);
    if (write_grp(path, s.n, grp)) fprintf(stderr, "skid: cannot write %s\n", path);
    wall_mark("grp");
    {
        float *gm = malloc(((size_t)nGroup + 1) * sizeof(float));
        float *gp = malloc(3 * ((size_t)nGroup + 1) * sizeof(float));
        float *gv = malloc(3 * ((size_t)nGroup + 1) * sizeof(float));
        float *grad = malloc(((size_t)nGroup + 1) * sizeof(float));
        for (int g = 1; g <= nGroup; ++g) {
            gm[g - 1] = gr[g].fMass;
            grad[g - 1] = gr[g].fRadius;
            for (int d = 0; d < 3; ++d) {
                gp[3 * (size_t)(g - 1) + d] = gr[g].rCenter[d];
                gv[3 * (size_t)(g - 1) + d] = gr[g].vcm[d];
            }
        }
        snprintf(path, sizeof(path), "%s.gtp", o.achName);
        if (tipsy_write_gtp(path, o.bStandard, s.time, nGroup, gm, gp, gv, grad))
            fprintf(stderr, "skid: cannot write %s\n", path);
        free(gm);
        free(gp);
        free(gv);
        free(grad);
    }
    if (o.bOutRay && moved) {
        int *flag = malloc((size_t)(s.n > 0 ? s.n : 1) * sizeof(int));
        for (int i = 0; i < s.n; ++i)
            flag[i] = moved[3 * (size_t)i] != s.pos[3 * (size_t)i] ||
                      moved[3 * (size_t)i + 1] != s.pos[3 * (size_t)i + 1] ||
                      moved[3 * (size_t)i + 2] != s.pos[3 * (size_t)i + 2];
        snprintf(path, sizeof(path), "%s.ray", o.achName);
        if (write_ray(path, &s, moved, flag, o.period)) fprintf(stderr, "skid: cannot write %s\n", path);
        free(flag);
    }
    if (o.bOutStats) {
        snprintf(path, sizeof(path), "%s.stat", o.achName);
        if (write_stats(path, &o, ctx, gr, nGroup)) fprintf(stderr, "skid: cannot write %s\n", path);
    }
    wall_mark("outputs");
    skid_timings t;
    die_on(skid_get_timings(ctx, &t), "skid_get_timings");
    printf("SKID GPU Time (device ms):\n");
    if (!o.bUnbindOnly) {
        printf("   Initial Density:    %.3f\n", t.density_ms);
        printf("   Moving Particles:   %.3f\n", t.moving_ms);
        printf("   Friends of Friends: %.3f\n", t.fof_ms);
        printf("   Microstepping:      %.3f\n", t.micro_ms);
    }
    if (!o.bNoUnbind) printf("   Unbinding:          %.3f\n", t.unbind_ms);
    fflush(stdout);
    free(grp);
    free(gr);
    free(moved);
    skid_destroy(ctx);
    tipsy_free(&s);
    wall_mark("teardown");
    if (g_wall) fprintf(stderr, "wall_abs_ms end %.3f\n", wall_ms());
    return 0;
}
