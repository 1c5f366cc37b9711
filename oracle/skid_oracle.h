/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * A single-threaded CPU restatement of skid's group-finding path
 * (N-BodyShop/skid v1.4.1).  It is the checker for the GPU library: only the
 * tests, the smoke check and bench.py's CPU-baseline leg call it.  The product
 * library never links or loads it.
 *
 * Semantics are the reference's, stated in an order-independent ("canonical")
 * form so that any correct implementation reproduces them:
 *
 *  - pair distance d2(q->c): float, no FMA, ((dx*dx + dy*dy) + dz*dz), with
 *    dx = fl(fl(xq + s*L) - xc) and s in {-1,0,1} the periodic image of the
 *    query nearest the candidate (kd.h:122-214, smooth1.c:72-75,104-107);
 *  - fBall2 = k-th smallest d2(i->j) over scatterers j, self included
 *    (smooth1.c:242-243); ties cannot change that value;
 *  - density: every pair (i, j in NN(i)) adds 1/2 m W(r, h_i) to both ends
 *    (smooth1.c:248-263), accumulated in FP64;
 *  - move field: for every live scatterer copy c (original or periodic
 *    replica, smooth1.c:283-332) and active mover y with d2(c->y) < b_c,
 *    a_y += m_c/(pi h_c^5) F(q) (x_c - y) (smooth1.c:447-459), FP64 sum;
 *  - friends-of-friends: edge iff d2(i->j) < tau^2 or d2(j->i) < tau^2
 *    (kd.c:869-876); groups numbered by ascending smallest member iOrder
 *    (the reference numbers them in tree discovery order, kd.c:840-847);
 *  - group reference point rel = position of the smallest-iOrder member
 *    (the reference uses the last member in its array order, kd.c:999-1001;
 *    any member gives the same centre up to rounding).
 *
 * Every array is indexed by iOrder unless stated otherwise.
 */
#ifndef SKID_ORACLE_H
#define SKID_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_DARK 1
#define OR_GAS 2
#define OR_STAR 4
#define OR_PLUMMER 1
#define OR_SPLINE 2

typedef struct or_params {
    float period[3];      /* FLT_MAX when not periodic (main.c:125-128) */
    float center[3];
    int   periodic;       /* -p given: periodic replica scatterers (main.c:279) */
    int   nSmooth;
    float fTau, fCvg, fScoop, fStep;
    float fDensMin, fTempMax, fMassMax;
    int   bGasAndDark, bGasOnly, bForceInitialCut;
    int   bNoScatterCut;  /* -nsp: no scatterer removal (README:29-30) */
    int   nMinMembers, nMaxMembers, bNoUnbind, iSoftType;
    int   bEps; float fEps;
    float G, Omega0, Lambda, fQuintess, H0, z;
    int   maxIter;        /* cap on outer move iterations; <=0 means none */
    int   verbose;        /* print the reference's progress lines */
    int   stopAfter;      /* 0 full run; 1 stop after group centres; 2 after unbinding */
} or_params;

typedef struct or_group {
    int   nMembers;
    float fMass;
    float rel[3], rCenter[3], rBound[3], vcm[3];
    float fRadius;
} or_group;

typedef struct or_result {
    int   nScatterInit;   /* scatter-active particles */
    int   nExtraScat;     /* periodic replica scatterers */
    int   nMove;
    int   nIter;          /* outer move iterations */
    int   nGroupFoF;      /* groups before unbinding, group 0 excluded */
    int   nUnbound;
    int   nGroup;         /* final groups, group 0 excluded */
    int   nScatFinal;
} or_result;

/* Stage functions (arrays of n points; pos is float[3n]). */
int or_knn_ball2(int n, const float *pos, int k, const float period[3],
                 float *ball2);
int or_knn_ball2_brute(int n, const float *pos, int k, const float period[3],
                       float *ball2);
int or_density(int n, const float *pos, const float *mass, const float *ball2,
               const float period[3], double *rho);
float or_d2(const float *q, const float *c, const float period[3]);

/* Move field at nm mover positions from ns scatterers (each with the
 * image-copy mask of its existing, live copies; bit 13 = the original). */
int or_replica_mask(int ns, const float *spos, const float *ball2,
                    const float period[3], const float center[3], int periodic,
                    unsigned int *exist_mask);
int or_field(int ns, const float *spos, const float *smass, const float *sball2,
             const unsigned int *alive_mask, int nm, const float *mpos,
             const float period[3], double *acc, double *absacc,
             unsigned int *touched_mask);

int or_fof(int n, const float *pos, const float period[3], float tau,
           const int *iorder, int *grp);

/* Whole pipeline (main.c:374-485 order).  grp[n] receives final group ids,
 * groups[] (capacity cap_groups, index 0 unused) the group records, rho[n]
 * the initial densities (0 for non-scatterers), moved[3n] the final mover
 * positions (input position for non-movers). */
int or_run(const or_params *par, int nGas, int nDark, int nStar, double time,
           const float *pos, const float *vel, const float *mass,
           const float *soft, const float *temp,
           int *grp, or_group *groups, int cap_groups, float *rho, float *ball2,
           float *moved, or_result *res);

/* Unbind-only mode: grp[n] (read and rewritten) holds the input group ids;
 * centers is NULL or 6 floats (rCenter, vcm) per group 1..max id. */
int or_run_unbind(const or_params *par, int nGas, int nDark, int nStar,
                  const float *pos, const float *vel, const float *mass,
                  const float *soft, int *grp, const float *centers,
                  or_group *groups, int cap_groups, or_result *res);

/* Unbinding of one group given its members (kd.c:1329-1460).  q arrays are in
 * the group's member order; returns the number of members left. */
int or_unbind_group(const or_params *par, int inType, int n,
                    float *qr, float *qv, float *qm, float *qs, int *qid,
                    double *pot, const float rel[3], float outVcm[3],
                    float *outMass, float outBound[3], int *removed_ids);

/* FP64 references for the adjoint checks.  Density: L = sum_i w_i rho_i
 * with the kNN sets (and k-th neighbours) of pos held fixed; for the nsel
 * particles sel[] the analytic gradient and central differences of step hfd
 * (3 doubles each) and the sum of |term| (one double each).  lists_ok = 0 if
 * some ball has no k-th neighbour at exactly fBall2 (returns -2). */
int or_density_adjoint_check(int n, const float *pos, const float *mass,
                             const float *w, int k, const float period[3],
                             int nsel, const int *sel, double hfd,
                             double *grad_an, double *grad_fd, double *absterm,
                             int *lists_ok);
/* The same, also with central differences of step hfd/2 (grad_fd_half,
 * may be NULL) for Richardson extrapolation. */
int or_density_adjoint_check2(int n, const float *pos, const float *mass,
                              const float *w, int k, const float period[3],
                              int nsel, const int *sel, double hfd,
                              double *grad_an, double *grad_fd,
                              double *grad_fd_half, double *absterm,
                              int *lists_ok);
/* Density field of ns scatterers at nq points: gradient, central
 * differences, sum of |term|. */
int or_field_grad_check(int ns, const float *spos, const float *smass,
                        const float *sball2, const float period[3], int nq,
                        const float *ypos, double hfd, double *grad_an,
                        double *grad_fd, double *absterm);

double or_exp2hub(double H0, double Omega0, double Lambda, double Quint,
                  double a);

#ifdef __cplusplus
}
#endif
#endif
