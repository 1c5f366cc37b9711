// The skid_ctx behind the opaque handle of include/skid_gpu.h.
#pragma once

#include "../../include/skid_gpu.h"
#include <cmath>

#include "internal.h"

namespace skid {

constexpr int PRUNE_STEPS = 5;   // main.c:13

// Device scalar slots (ints) in ctx->d_scal.
enum {
    SC_WORK = 0,     // work-queue counter of tree walks
    SC_STATUS = 1,   // latched status bits
    SC_NC = 2,       // live scatterer copies
    SC_NC2 = 3,
    SC_FLOOR = 4,
    SC_DIRTY = 5,
    SC_NA = 6,
    SC_NA2 = 7,
    SC_EXTRA = 8,
    SC_NG = 9,       // groups
    SC_NG2 = 10,
    SC_NUNB = 11,    // particles unbound
    SC_WORK2 = 12,
    SC_DONE = 13,    // finished blocks of the copy write-back (last one publishes)
    SC_COUNT = 32
};

enum Stage {
    STAGE_NONE = 0,
    STAGE_LOADED,
    STAGE_SCATTER,
    STAGE_DENSITY,
    STAGE_MOVE,
    STAGE_FOF,
    STAGE_GROUPS,
    STAGE_UNBOUND,
    STAGE_FINAL
};

struct Ranges {
    int start[3], len[3], n;
};

float float_floor(double t);

#define CK(x)                                               \
    do {                                                    \
        cudaError_t e__ = (x);                              \
        if (e__ != cudaSuccess) return ctx->fail_cuda(e__); \
    } while (0)

// Group state (sized by the number of groups).
struct GroupState {
    int nGroup = 0;                 // including group 0
    DBuf<int> start, count;         // member range per group in `members`
    DBuf<int> members;              // iOrder, grouped, ascending iOrder inside a group
    DBuf<int> gof;                  // group of each member slot
    DBuf<skid_group> rec;           // per group record
    DBuf<double> sums;              // per group FP64 sums
    DBuf<int> map;                  // too-small remap
    DBuf<int> gtmp, gtmp2;
    DBuf<skid_group> rec2;
};

struct UnbindParams {
    float3 period;
    bool per;
    float fScoop;
    int nmax;          // -maxgroup
    float G, a, aH, opz, z;
    float scale;       // 2^S of the fixed-point potentials
    int plummer, subpot, nounbind;
    int n;             // particles (size of grp)
    int tw, bs;        // removal schedule: warp-per-group up to tw members, blocks of bs
                       // threads above; -1 = autotuned
    int clu_min;       // the largest groups above this many members may take a block cluster (0: none)
    bool clu_auto;     // clu_min is the default: only a tuned schedule that measured them faster uses clusters
    bool per_group;    // one potential and one removal launch per group
};

struct UnbindScratch {
    DBuf<float4> qr, qv, slist;
    DBuf<float4> qw;                 // large groups: (a v + aH r, softening) per member
    DBuf<long long> pot, pot_save;
    DBuf<int> qid, scnt, soff, nt, toff, cnt, grp_save;
    DBuf<uint32_t> order;
    DBuf<int2> items;
    DBuf<float> ssoft, usoft;
    DBuf<skid_group> rec_save;
    int tuned_tw = -1, tuned_bs = -1;   // autotuned removal schedule (kept per context)
    int tuned_cs = -1;                  // autotuned: the largest groups on block clusters (1) or not (0)
    int used_tw = -1, used_bs = -1;     // schedule of the last run
    int used_cs = 1, used_nclu = 0;     // cluster size and clustered groups of the last run
    float tune_ms[32] = {};
    int ntune = 0, ntune_now = 0;
    float pot_ms = 0.0f, remove_ms = 0.0f;   // last run (CUDA events)
};

// fof.cu
cudaError_t fof_run(Tree &t, const float4 *pts, int np, const int *mio, int niorder, float tau,
                    float3 L, bool per, SortScratch &ss, DBuf<int> &par, DBuf<int> &minio,
                    DBuf<int> &flag, int *grp, int *d_ng, int *d_work, unsigned *d_status,
                    cudaStream_t st);
// groups.cu
cudaError_t group_order(const int *grp, int n, int ng, SortScratch &ss, GroupState &G,
                        cudaStream_t st);
cudaError_t group_props(GroupState &G, const float4 *pos4, const float4 *vel4, const float4 *moved,
                        float3 L, float3 wrapHi, float3 wrapLo, bool com, bool rel_last,
                        cudaStream_t st);
cudaError_t too_small(GroupState &G, int *grp, int n, int nmin, int *d_ng, SortScratch &ss,
                      cudaStream_t st);
cudaError_t group_radius(GroupState &G, const int *grp, int n, const float4 *pos4, float3 L,
                         cudaStream_t st);
// adjoint.cu
struct AdjointState {
    DBuf<float> win;            // cotangent by iOrder (or per query point)
    DBuf<float> w, g, out;      // cotangent (tree order), gradient (tree order), gradient by iOrder
    DBuf<int> nbr, ncnt;        // stored ball lists, `cap` per scatterer
    int cap = 0;
    bool lists = false;         // lists match the current density
    DBuf<int2> items;           // potential work items (selection slot, tile)
    DBuf<int> gsel;
    DBuf<float> v;
    DBuf<double> E;
};
cudaError_t density_adjoint(const Tree &t, const float *ball2_sorted, const int *sidx, const float *w_io,
                            int n_io, float3 L, bool per, int mode, int k, AdjointState &A,
                            int *d_work, unsigned *d_status, cudaStream_t st);
cudaError_t potential_adjoint(const GroupState &G, const float4 *pos4, const float4 *vel4, int n,
                              float3 period, float Gc, int plummer, int nSel, const int *h_sel,
                              const float *h_v, bool want_grad, AdjointState &A, cudaStream_t st);
// unbind.cu
cudaError_t unbind_run(GroupState &G, const int *gof, int nslots, const float4 *pos4,
                       const float4 *vel4, Tree &ut, const UnbindParams &P, int *grp,
                       int *d_unbound, SortScratch &ss, UnbindScratch &U, cudaStream_t st);

}  // namespace skid

struct skid_ctx {
    skid_params par{};
    float3 L{}, hL{};
    bool per = false;
    cudaStream_t st = nullptr;
    int *d_scal = nullptr;
    unsigned *d_status = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    int n = 0, nGas = 0, nDark = 0, nStar = 0, inType = 0;
    double time = 0.0;
    double mass_total = 0.0;        // host copy, for the fixed-point potential scale
    float soft_min = 0.0f;
    float soft_min_input = 0.0f;
    skid::DBuf<double> ms_dev;      // device reduction: [MS_BLOCKS partials x 2], then (sum |m|, min soft)
    bool ms_pending = false;        // mass_total / soft_min_input not yet read back
    int stage = skid::STAGE_NONE;
    int last_error = 0;
    int last_cuda = 0;              // first CUDA runtime error seen

    // particles by iOrder
    skid::DBuf<float4> pos4, vel4;
    skid::DBuf<float> temp, rho, rho_final, ball2, raw;
    skid::DBuf<float> soft_orig;    // input softening, kept once -e overrides it
    bool soft_changed = false;
    skid::DBuf<int> grp;

    // scatterers, movers, groups
    skid::Ranges ranges{};
    int nScatInit = 0, nExtraScat = 0;
    skid::Tree stree;               // periodic tree over the scatterers (kNN, density)
    skid::DBuf<float4> spos0;       // scatterers in list order (tree input)
    skid::DBuf<int> sidx0, sidx;    // iOrder in list / tree order
    skid::DBuf<float> sb2, srho;    // fBall2 and density in tree order
    skid::DBuf<float4> saux;        // density-gather node data
    skid::CopyState C;              // move-phase scatterer copies
    skid::Tree ctree;               // tree over the copies (ball boxes)
    int nCopies = 0;
    int nMove = 0, nActive = 0;
    skid::MoverState M;
    skid::Tree mtree;               // tree over movers (FoF)
    skid::DBuf<int> parent;         // union-find
    skid::GroupState G;
    skid::Tree utree;               // tree over ungrouped particles (scoop)
    skid::UnbindScratch U;
    skid::DBuf<int> fof_minio, fof_flag;
    skid::DBuf<float4> moved4;      // moved positions by iOrder
    skid::SortScratch ss;
    skid::DBuf<float> knn_heap;     // kNN heaps when k is too large for shared memory
    skid::AdjointState adj;         // density / potential adjoints

    // outer-iteration CUDA graphs, one per movers-per-warp setting
    static constexpr int NSLOT = 6;          // movers per warp 32, 16, 8, 4, 1, 64
    cudaGraphExec_t iter_graph[NSLOT] = {};
    long long iter_graph_kernels[NSLOT] = {};
    float g_fStep[NSLOT] = {}, g_fCvg[NSLOT] = {};
    bool g_nocut[NSLOT] = {};
    bool g_stats[NSLOT] = {};
    int g_bound[NSLOT] = {};                 // active movers the graph's prune is sized for
    // What else a captured iteration bakes in: the buffers (allocation
    // epoch), the copy tree's shape, the mover and copy counts and the
    // movers' Hilbert key frame.  A graph whose key still matches is replayed
    // in later runs instead of being captured again.
    struct GraphKey {
        unsigned long long epoch = 0;
        int leafBase = 0, nMove = 0, nScat = 0, nExtra = 0, n = 0;
        float klo[3] = {}, kinv[3] = {};
        bool unfused = false;
        bool operator==(const GraphKey &o) const
        {
            return epoch == o.epoch && leafBase == o.leafBase && nMove == o.nMove &&
                   nScat == o.nScat && nExtra == o.nExtra && n == o.n && klo[0] == o.klo[0] &&
                   klo[1] == o.klo[1] && klo[2] == o.klo[2] && kinv[0] == o.kinv[0] &&
                   kinv[1] == o.kinv[1] && kinv[2] == o.kinv[2] && unfused == o.unfused;
        }
    };
    GraphKey g_key[NSLOT];
    GraphKey graph_key() const
    {
        GraphKey k;
        k.epoch = skid::alloc_epoch();
        k.leafBase = ctree.leafBase;
        k.nMove = nMove;
        k.nScat = nScatInit;
        k.nExtra = nExtraScat;
        k.n = n;
        k.klo[0] = mkey_lo.x; k.klo[1] = mkey_lo.y; k.klo[2] = mkey_lo.z;
        k.kinv[0] = mkey_inv.x; k.kinv[1] = mkey_inv.y; k.kinv[2] = mkey_inv.z;
        k.unfused = opt_field_unfused;
        return k;
    }
    float3 mkey_lo{}, mkey_inv{};   // Hilbert key frame of mover positions
    // move-field kernel timing: an event pair per step slot of an iteration
    cudaEvent_t fev[2 * skid::PRUNE_STEPS] = {};
    double *d_fbytes = nullptr;     // [bytes, launches] accumulated on device
    unsigned long long *d_fstats = nullptr;   // move-field work counters
    bool field_stats_on = false;
    bool iter_eager_done = false;

    // probes
    skid::Tree probe_tree;
    skid::DBuf<float> probe_f, probe_acc;
    skid::DBuf<float4> probe_p4;
    skid::DBuf<int> probe_i, probe_i2;
    skid::DBuf<unsigned char> probe_t;
    skid::DBuf<uint32_t> tipsy_raw;   // TIPSY record words as read (skid_set_tipsy)
    skid::DBuf<int> stat_start;      // .stat: first sorted slot of each group
    skid::DBuf<skid_stat> stat_out;  // .stat: per-group columns
    skid::DBuf<float> split_acc;     // field parts of split movers
    skid::DBuf<int> split_cnt;       // parts finished per split mover (zero between steps)

    skid_timings tim{};
    long long gather_launches = 0, kernel_launches = 0;

    int fail(int code);
    int fail_cuda(cudaError_t e);
    int sync_check();
    int read_int(const int *d, int *h);
    void timer_start();
    float timer_stop();
    skid::FieldArgs field_args(float fStep, bool initial, float *acc_out);
    float3 wrap_hi() const;
    float3 wrap_lo() const;

    // 2^S such that |potential| * 2^S < 2^62: the spline potential is at most
    // 1.4 * 2/(eps_i+eps_j) <= 1.4/eps_min per unit G*mass (grav.h:11-31), and
    // the Plummer form at most 2/(eps_i+eps_j).
    // The input's total |mass| and smallest softening, reduced on the device
    // when the particles were set; read back here the first time they are
    // needed.
    int ensure_mass_soft()
    {
        if (!ms_pending) return 0;
        double v[2];
        if (cudaMemcpyAsync(v, ms_dev.p, sizeof(v), cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st))
            return -1;
        mass_total = v[0];
        soft_min_input = (float)v[1];
        if (!soft_changed) soft_min = soft_min_input;
        ms_pending = false;
        return 0;
    }
    float pot_scale(float G) const
    {
        if (!(soft_min > 0.0f)) return ldexpf(1.0f, 40);
        double B = 4.0 * fabs((double)G) * mass_total * 1.4 / (double)soft_min;
        int S = (int)floor(62.0 - log2(B > 1e-300 ? B : 1e-300));
        if (S < 0) S = 0;
        if (S > 60) S = 60;
        return ldexpf(1.0f, S);
    }
    int enqueue_step(float fStep, bool initial, bool nocut, int slot, int G, bool compact = true);
    // Crossovers measured on GB300 with the 2^21-particle workload: per-step
    // move-field time is lowest with 32 movers per warp above ~600k active
    // movers, 16 down to ~400k, 8 down to ~50k, 4 down to ~25k, one below.
    int opt_G = 0, opt_g32_min = 600000, opt_g16_min = 400000, opt_g8_min = 100000, opt_g4_min = 30000;
    int opt_g64_min = 0;                          // 64 movers per warp at or above (0: never)
    int opt_curve = 7;                            // Hilbert order (else Morton) of: 1 movers, 2 copies, 4 scatterer tree
    int opt_unbind_tw = -1, opt_unbind_bs = -1;   // -1: autotuned on the first skid_unbind
    int opt_unbind_clu_min = -1;                  // the largest groups above it may take a block cluster; 0 = never;
                                                  // -1 = 2048, and only where the tuner measured clusters faster
    bool opt_unbind_per_group = false;
    bool opt_field_unfused = false;                // field pass and move pass as separate kernels
    skid::DBuf<float> unfused_acc;
    // Largest active count that selects G (the prune of an iteration graph
    // for G is sized for it; the count only falls within a run).
    int slot_bound(int G) const
    {
        int b = opt_G || G == 64 || (G == 32 && !opt_g64_min) ? M.cap
                : G == 32        ? opt_g64_min
                : G == 16        ? opt_g32_min
                : G == 8         ? opt_g16_min
                : G == 4         ? opt_g8_min
                                 : opt_g4_min;
        if (b < nActive) b = nActive;
        return b < M.cap ? b : M.cap;
    }
    int movers_per_warp() const
    {
        if (opt_G) return opt_G;
        return opt_g64_min && nActive >= opt_g64_min ? 64
               : nActive >= opt_g32_min ? 32
               : nActive >= opt_g16_min ? 16
               : nActive >= opt_g8_min  ? 8
               : nActive >= opt_g4_min  ? 4
                                        : 1;
    }
    void drop_graphs()
    {
        std::lock_guard<std::recursive_mutex> lk(skid::device_mutex());
        for (auto &g : iter_graph)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    void collect_field_times(int nslots);

    unsigned char *probe_touched()
    {
        size_t need = C.cap > 0 ? C.cap : 1;
        if (skid::dalloc(probe_t, need)) return nullptr;
        return probe_t.p;
    }

    void reset_pipeline()
    {
        // the move-iteration graphs stay: skid_move_iterate replays one only
        // while its key (graph_key) still matches
        iter_eager_done = false;
        stage = skid::STAGE_NONE;
        nScatInit = nExtraScat = nMove = nActive = 0;
        G.nGroup = 0;
        adj.lists = false;
        tim = skid_timings{};
        cudaMemsetAsync(d_scal, 0, skid::SC_COUNT * sizeof(int), st);
        cudaMemsetAsync(d_fbytes, 0, 2 * sizeof(double), st);
    }

    int alloc_particles(int np)
    {
        using skid::dalloc;
        size_t m = np > 0 ? np : 1;
        if (dalloc(pos4, m) || dalloc(vel4, m) || dalloc(temp, m) || dalloc(rho, m) ||
            dalloc(rho_final, m) || dalloc(ball2, m) || dalloc(grp, m) || dalloc(raw, 9 * m))
            return -1;
        return 0;
    }

    int alloc_scatterers(int ns)
    {
        using skid::dalloc;
        size_t m = ns > 0 ? ns : 1;
        if (dalloc(spos0, m) || dalloc(sidx0, m) || dalloc(sidx, m) || dalloc(sb2, m) ||
            dalloc(srho, m) || dalloc(saux, m))
            return -1;
        return 0;
    }

    int alloc_movers(int nm)
    {
        using skid::dalloc;
        size_t m = nm > 0 ? nm : 1;
        if (dalloc(M.mpos, m) || dalloc(M.mold, m) || dalloc(M.mio, m) || dalloc(M.act, m) ||
            dalloc(M.act2, m) || dalloc(M.keep, m) || dalloc(M.kpos, m))
            return -1;
        if (!split_cnt.p) {
            // split one-mover-per-warp steps: partial fields and part counters
            if (dalloc(split_acc, 3 * (size_t)skid::FIELD_SPLIT_CAP) ||
                dalloc(split_cnt, skid::FIELD_SPLIT_CAP))
                return -1;
            if (cudaMemsetAsync(split_cnt.p, 0, skid::FIELD_SPLIT_CAP * sizeof(int), st)) return -1;
        }
        M.cap = (int)m;
        return 0;
    }

    ~skid_ctx()
    {
        using skid::dfree;
        drop_graphs();
        dfree(pos4); dfree(vel4); dfree(temp); dfree(rho); dfree(rho_final); dfree(ball2);
        dfree(raw); dfree(grp); dfree(soft_orig);
        for (skid::Tree *t : {&stree, &ctree, &mtree, &utree, &probe_tree}) {
            dfree(t->pos); dfree(t->perm); dfree(t->lo); dfree(t->hi); dfree(t->blo);
            dfree(t->bhi); dfree(t->flag);
        }
        dfree(spos0); dfree(sidx0); dfree(sidx); dfree(sb2); dfree(srho); dfree(saux);
        dfree(C.cpos); dfree(C.ccoef); dfree(C.cpos2); dfree(C.ccoef2); dfree(C.touched);
        dfree(C.keep); dfree(C.kpos); dfree(C.mask); dfree(C.cnt); dfree(C.off);
        dfree(M.mpos); dfree(M.mold); dfree(M.mio); dfree(M.act); dfree(M.act2); dfree(M.keep);
        dfree(M.kpos);
        dfree(parent);
        dfree(G.start); dfree(G.count); dfree(G.members); dfree(G.rec); dfree(G.sums);
        dfree(G.map); dfree(G.gtmp); dfree(G.gtmp2); dfree(G.gof); dfree(G.rec2);
        dfree(U.qr); dfree(U.qv); dfree(U.qw); dfree(U.slist); dfree(U.pot); dfree(U.qid); dfree(U.scnt);
        dfree(U.soff); dfree(U.nt); dfree(U.toff); dfree(U.cnt); dfree(U.items); dfree(U.ssoft);
        dfree(unfused_acc);
        dfree(U.usoft); dfree(U.pot_save); dfree(U.grp_save); dfree(U.order); dfree(U.rec_save);
        dfree(fof_minio); dfree(fof_flag); dfree(moved4);
        dfree(ss.k0); dfree(ss.k1); dfree(ss.v0); dfree(ss.v1); dfree(ss.hist); dfree(ss.glob); dfree(ss.blk);
        dfree(ss.box);
        dfree(probe_f); dfree(probe_acc); dfree(probe_p4); dfree(probe_i); dfree(probe_i2);
        dfree(probe_t); dfree(stat_start); dfree(stat_out); dfree(tipsy_raw); dfree(knn_heap); dfree(split_acc); dfree(split_cnt); dfree(ms_dev);
        dfree(adj.win); dfree(adj.w); dfree(adj.g); dfree(adj.out); dfree(adj.nbr); dfree(adj.ncnt);
        dfree(adj.items); dfree(adj.gsel); dfree(adj.v); dfree(adj.E);
        std::lock_guard<std::recursive_mutex> lk(skid::device_mutex());
        if (d_scal) cudaFree(d_scal);
        if (d_fbytes) cudaFree(d_fbytes);
        if (d_fstats) cudaFree(d_fstats);
        for (cudaEvent_t &e : fev)
            if (e) cudaEventDestroy(e);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (st) cudaStreamDestroy(st);
    }
};
