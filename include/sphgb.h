/* sphgb: C ABI of the GB300-native single-rank SPH hydro sweep (sm_103a).
 *
 * Every entry point returns an sphgb_status (0 = success); no C++ exception crosses it.
 * Pointers inside sphgb_particles are DEVICE pointers owned by the caller, exactly like the
 * DeviceVector fields of the reference's DeviceParticlesData
 * (sph/include/sph/particles_data_gpu.cuh:76-104).  The context owns everything else: sort
 * scratch, the cornerstone tree, the octree, the neighbour lists and the kernel tables.
 * All work is enqueued on the context's stream; a call returns once its results are ready
 * unless noted.
 *
 * Two precisions share one set of entry points:
 *   SPHGB_FP64   every field is double (the reference with HydroType=XM1Type=Tmass=double);
 *   SPHGB_MIXED  the reference's default SphTypes (sph/include/sph/types.hpp:39-46): x,y,z,u,du
 *                double, every other hydro field float.  Pair arithmetic runs in FP32 on
 *                grid-local coordinate offsets; keys and neighbour tests stay exact FP64.
 */
#ifndef SPHGB_H
#define SPHGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SPHGB_OK = 0,
    SPHGB_ERR_ARG = 1,        /* invalid argument (null pointer, size, range) */
    SPHGB_ERR_CUDA = 2,       /* a CUDA runtime call failed; sphgb_last_cuda_error() tells which */
    SPHGB_ERR_ALLOC = 3,      /* device allocation failed */
    SPHGB_ERR_STATE = 4,      /* call out of order (e.g. pair pass before neighbours) */
    SPHGB_ERR_TRAVERSAL = 5,  /* octree traversal stack overflow (reference: 0xFFFFFFFF stack flag) */
    SPHGB_ERR_NOCONV = 6,     /* h / neighbour-count iteration did not converge for some particles */
    SPHGB_ERR_NOTFOUND = 7,   /* no CUDA device / extension not usable */
    SPHGB_ERR_TOO_LARGE = 8,  /* request exceeds a fixed capacity */
    SPHGB_ERR_INPUT = 9,      /* a coordinate, h or box limit is not finite, or h <= 0; found by a check
                                 pass before any key, tree or search kernel runs on the data */
    SPHGB_ERR_TIMEOUT = 10    /* a bounded device-side wait gave up (the radix sort's look-back between
                                 tiles); the results of that call are invalid, the context stays usable */
} sphgb_status;

typedef enum { SPHGB_FP64 = 0, SPHGB_MIXED = 1 } sphgb_precision;
/* cstone::BoundaryType (domain/include/cstone/sfc/box.hpp:80-85); fixed boundaries act as open in
 * the key, tree and pair passes and freeze resting particles next to them in the position update */
typedef enum { SPHGB_BC_OPEN = 0, SPHGB_BC_PERIODIC = 1, SPHGB_BC_FIXED = 2 } sphgb_boundary;
typedef enum { SPHGB_STD = 0, SPHGB_VE = 1 } sphgb_variant;

typedef struct sphgb_ctx sphgb_ctx;

/* cstone::Box (domain/include/cstone/sfc/box.hpp:94-174): limits and boundary types */
typedef struct {
    double lim[6];            /* xmin xmax ymin ymax zmin zmax */
    uint8_t bc[3];            /* sphgb_boundary per dimension */
} sphgb_box;

/* Physics constants of sphexa::ParticlesData (sph/include/sph/particles_data.hpp:90-146) */
typedef struct {
    uint32_t ng0;             /* target neighbour count, default 100 */
    uint32_t ngmax;           /* neighbour cap, default 150 */
    uint32_t bucket;          /* leaf bucket size of the cornerstone tree, default 64 */
    double gamma;             /* adiabatic index, default 5/3 */
    double Kcour;             /* Courant factor, default 0.2 */
    double sincIndex;         /* sinc kernel exponent, default 6 */
    double alphamin, alphamax, decay_constant;  /* AV switch, defaults 0.05, 1.0, 0.2 */
    double minDt;             /* d.minDt seen by the AV-switch decay */
} sphgb_params;

/* Field pointers of one particle set (device memory, caller-owned).  double* fields are FP64
 * in both precisions; void* fields are double (SPHGB_FP64) or float (SPHGB_MIXED). */
typedef struct {
    int64_t n;
    int32_t precision;        /* sphgb_precision */
    uint64_t* keys;           /* optional: receives the sorted SFC keys */
    double *x, *y, *z, *u, *du;
    void *h, *m, *vx, *vy, *vz, *alpha;
    void *rho, *p, *c, *xm, *kx, *gradh, *prho, *divv, *curlv;
    void *c11, *c12, *c13, *c22, *c23, *c33;
    void *ax, *ay, *az;
    void *dV11, *dV12, *dV13, *dV22, *dV23, *dV33;
    uint32_t* nc;             /* neighbour count incl. self (sphexa nc field) */
} sphgb_particles;

typedef struct {
    int64_t num_leaves, num_nodes, num_internal;
    int32_t level_range[23];
    int64_t nc_sum;           /* sum over targets of min(nc-1, ngmax) */
    uint32_t nc_max;          /* max nc (incl. self) */
    int64_t capped;           /* particles with nc - 1 > ngmax */
    int64_t h_iterations;     /* h-iteration rounds run by the last neighbour search */
    int64_t h_fails;          /* particles that hit the 10-iteration limit */
    int64_t candidates;       /* candidate pairs tested by the last neighbour search */
    int64_t fp64_rechecks;    /* candidate pairs that needed the exact FP64 test */
    int64_t refined_gradh;    /* mixed form: particles whose gradh was recomputed in FP64 (last pass) */
    int64_t refined_divv;     /* mixed form: particles whose divv sign was settled in FP64 (last pass) */
} sphgb_stats;

/* ---- context ---- */
const char* sphgb_status_string(int status);
const char* sphgb_last_cuda_error(void);
int sphgb_version(void);
/* create a context on `device`; stream 0 = the legacy default stream */
int sphgb_create(sphgb_ctx** ctx, int device);
int sphgb_destroy(sphgb_ctx* ctx);
int sphgb_set_stream(sphgb_ctx* ctx, void* cuda_stream);
int sphgb_set_params(sphgb_ctx* ctx, const sphgb_params* params);
/* Summation order of the FP64 VE passes xmass, gradh, IAD + divv/curlv, AV switches and
 * momentum-energy (no reference counterpart; the reference's GPU passes are order-fixed, e.g.
 * hydro_ve/momentum_energy_gpu.cu:53-144).  on = 0 (default): when the lists cover every particle,
 * each pair whose two ends list each other is evaluated once and the neighbour's share is added
 * with FP64 atomics, so the last bits of those passes' outputs can differ from run to run.
 * on = 1: every list owner sums its own pairs in list order, bitwise reproducible. */
int sphgb_set_deterministic(sphgb_ctx* ctx, int32_t on);
/* Forward tape of the VE adjoint (no reference counterpart).  on = 1: the FP64 VE passes over all
 * particles (gradh, IAD + divv/curlv, AV switches, momentum-energy) keep the per-particle sums
 * that sphgb_adjoint_ve needs (16 doubles per particle, held by the context), and the adjoint
 * reads them instead of summing them again over the lists.  The tape belongs to the neighbour
 * lists it was written on; a later neighbour search invalidates it.  on = 0 (default) frees it. */
int sphgb_set_adjoint_tape(sphgb_ctx* ctx, int32_t on);
/* Mixed form only (no reference counterpart): on = 1 (default) recomputes in FP64, from the exact
 * inputs, the particles whose gradh is near 0 (|gradh| < 0.1) or whose divv sign lies within the
 * FP32 error bound, with the neighbour shells their values depend on; on = 0 leaves the FP32
 * results.  The counts of the last sweep are in sphgb_stats.refined_gradh / refined_divv. */
int sphgb_set_mixed_refinement(sphgb_ctx* ctx, int32_t on);
/* Form of the kernel function W(v) and dW/dv in the FP64 pair passes and the FP64 adjoints (no
 * reference counterpart).  SPHGB_KERNEL_TABLE (default): the reference's linear interpolant of its
 * 20000-entry tables (sph/include/sph/table_lookup.hpp:10-26), whose slope jumps at every node
 * (every 1e-4 in v).  SPHGB_KERNEL_SMOOTH: a cubic Hermite piece on each of the same intervals
 * through the closed-form values and derivatives of sinc^n (sph_kernel_tables.hpp:77-157) at both
 * nodes, so W and dW/dv are continuously differentiable and central differences of the forward
 * passes converge to the adjoint's gradient; results differ from the table form by the table's
 * interpolation error (within 2e-8 of
 * the maximum of W and of |dW/dv|).  The mixed passes always use their own cubic pieces. */
typedef enum { SPHGB_KERNEL_TABLE = 0, SPHGB_KERNEL_SMOOTH = 1 } sphgb_kernel_form;
int sphgb_set_kernel_form(sphgb_ctx* ctx, int32_t form);
/* Domain mode.  0 (default): every sphgb_domain_sync stands alone (open dimensions take the
 * particle extrema).  1: the syncs are the steps of one simulation, as cstone::Domain::sync
 * (domain/include/cstone/domain/assignment.hpp:80-82): from the second sync on, the open-dimension
 * box follows limitBoxShrinking (box.hpp:397-414) against the previous sync's box, and the tree is
 * the reference's single-rank focus tree: converged at the first sync, then updated once per sync
 * from the previous tree and the previous sync's counts (focus/octree_focus_mpi.hpp:88-253,
 * domain/domain.hpp:199-211), so a leaf may hold more than bucket particles until the next sync
 * splits it.  Setting the mode starts a new sequence.  Mode 0 builds the converged tree every sync. */
int sphgb_set_domain_mode(sphgb_ctx* ctx, int32_t mode);
int sphgb_default_params(sphgb_params* params);
/* kernel normalisation constant K used by the pair passes */
int sphgb_get_kernel_K(sphgb_ctx* ctx, double* K);

/* ---- domain: replaces Domain<KeyType,T,GpuTag>::sync + octreeProperties at one rank
 *      (domain/include/cstone/domain/domain.hpp:181-234, 416-428).  Fits open box limits
 *      (sfc/box_mpi.hpp:68-103), computes Hilbert keys (sfc/sfc.hpp:267-275), stable-sorts by
 *      key (primitives/gather.cuh:50-76), permutes every non-null field of `p` in place, and
 *      builds the cornerstone tree with bucket `params.bucket` (tree/csarray.hpp:429-440), the
 *      internal octree (tree/octree.hpp:136-157) and the leaf layout.  `box` is in/out. */
int sphgb_domain_sync(sphgb_ctx* ctx, sphgb_particles* p, sphgb_box* box);
/* device pointers of the tree built by the last sync (valid until the next sync) */
int sphgb_get_tree(sphgb_ctx* ctx, const uint64_t** leaves, const uint32_t** layout,
                   const uint64_t** prefixes, const int32_t** child_offsets,
                   const int32_t** internal_to_leaf, sphgb_stats* stats);
/* cstone::OctreeNsView (domain/include/cstone/tree/octree.hpp:279-300) of the tree built by the
 * last sync, as cstone::Domain::octreeProperties returns it (domain/include/cstone/domain/domain.hpp:
 * 416-428): device pointers, valid until the next sync */
typedef struct {
    int64_t num_leaf_nodes, num_nodes, num_internal;
    const uint64_t* prefixes;        /* node keys with the placeholder bit, level-major order */
    const int32_t* child_offsets;    /* first child of each node, 0 for a leaf */
    const int32_t* internal_to_leaf; /* leaf index of each leaf node (the reference's labels otherwise) */
    const int32_t* level_range;      /* 23 entries: first node of each level */
    const uint64_t* leaves;          /* cornerstone leaf keys, num_leaf_nodes + 1 entries */
    const uint32_t* layout;          /* first particle of each leaf, num_leaf_nodes + 1 entries */
    const double* centers;           /* geometric node centers x y z (focus/source_center.hpp:129-141) */
    const double* sizes;             /* geometric node half sizes x y z (sfc/box.hpp:317-334) */
    int32_t max_depth;               /* deepest level that holds a node */
} sphgb_octree_view;
int sphgb_get_octree_view(sphgb_ctx* ctx, sphgb_octree_view* view);
/* the parameters in force (the values sphgb_set_params stored) */
int sphgb_get_params(sphgb_ctx* ctx, sphgb_params* params);
/* sph::computeGroups / computeSpatialGroups on the GPU (sph/include/sph/groups.hpp:41-56,
 * domain/include/cstone/traversal/groups_gpu.cu:58-135): the target groups of this library's pair
 * passes are the runs of 32 SFC-consecutive particles of [first, last), one warp each.  Writes
 * *num_groups = ceil((last - first) / 32) and, when `splits` is non-null, the num_groups + 1 group
 * boundaries first, first + 32, ..., last into splits (device, `capacity` entries), so that
 * groupStart = splits and groupEnd = splits + 1 as in cstone::GroupData (traversal/groups.hpp:37-52).
 * groupDt of sphgb_compute_momentum_energy is indexed by these groups. */
int sphgb_target_groups(sphgb_ctx* ctx, int64_t first, int64_t last, uint32_t* splits, int64_t capacity,
                        int64_t* num_groups);
/* sorted order of the last sync: order[i] = pre-sync index of sorted particle i (device) */
int sphgb_get_order(sphgb_ctx* ctx, const uint32_t** order);
/* permute one more per-particle field (device, n elements of elem_bytes = 1, 2, 4 or 8) into the
 * order of the last sync, in place: the reference's sync reorders every property it is handed
 * (domain/include/cstone/domain/domain.hpp:533-595); sphgb_domain_sync reorders the fields of
 * sphgb_particles, this call the rest (x_m1, du_m1, temp, ...) */
int sphgb_apply_order(sphgb_ctx* ctx, void* field, int32_t elem_bytes);
/* stable sort of n 64-bit keys by their bits [0, end_bit) with optional 32-bit values, device
 * pointers, out of place (keys_in and vals_in are left as they are): the GPU sortByKeyGpu of the
 * reference (domain/include/cstone/primitives/primitives_gpu.cu:323-340), the sort behind every
 * sync.  vals_in and vals_out are both null or both set; 1 <= end_bit <= 64, n < 2^32.  The
 * context keeps the scratch.  Synchronises the context's stream; SPHGB_ERR_TIMEOUT if a
 * look-back wait between tiles gave up (the output is then invalid). */
int sphgb_sort_by_key(sphgb_ctx* ctx, const uint64_t* keys_in, uint64_t* keys_out, const uint32_t* vals_in,
                      uint32_t* vals_out, int64_t n, int32_t end_bit);

/* ---- neighbours ---- */
/* cstone::findNeighbors (domain/include/cstone/findneighbors.hpp:149-170): fixed h, no
 * iteration.  Writes neighbors[(i-first)*ngmax + k] (reference layout, device) when non-null
 * and nc[i-first] = neighbour count EXCLUDING self, like the reference.  Lists are sorted
 * ascending; a particle with more than ngmax neighbours keeps its ngmax smallest indices. */
int sphgb_find_neighbors(sphgb_ctx* ctx, const double* x, const double* y, const double* z, const void* h,
                         int32_t h_precision, int64_t first, int64_t last, uint32_t ngmax, uint32_t* neighbors,
                         uint32_t* nc);
/* sph::findNeighborsSfc / findNeighborsSph (sph/include/sph/find_neighbors.hpp:10-56): builds
 * the context's neighbour lists for [first,last) with the coupled h / nc iteration (at most 10
 * rounds), writes p->nc (incl. self) and may update p->h.  Returns SPHGB_ERR_NOCONV (a warning:
 * the lists are complete) when some particles did not converge, as the reference prints. */
int sphgb_find_neighbors_sph(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* copy the context's lists out in the reference CPU layout neighbors[(i-first)*ngmax + k] */
int sphgb_export_neighbors(sphgb_ctx* ctx, uint32_t* neighbors_device);

/* ---- pair passes, each (GroupView{first,last}, Dataset&, Box) like the reference ---- */
/* sph::computeDensity (sph/include/sph/hydro_std/density.hpp:55-60) -> rho */
int sphgb_compute_density(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeEOS_HydroStd, ideal gas (hydro_std/eos.hpp:147-152) -> p, c */
int sphgb_compute_eos_std(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeIAD (hydro_std/iad.hpp:74-79) -> c11..c33 */
int sphgb_compute_iad(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeMomentumEnergySTD (hydro_std/momentum_energy.hpp:96-101) -> ax ay az du; Courant
 * dt minimum to *minDtCourant (d.minDtCourant) when non-null */
int sphgb_compute_momentum_energy_std(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last,
                                      double* minDtCourant);
/* sph::computeXMass (hydro_ve/xmass.hpp:69-74) -> xm */
int sphgb_compute_xmass(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeVeDefGradh (hydro_ve/ve_def_gradh.hpp:80-85) -> kx, gradh */
int sphgb_compute_ve_def_gradh(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeEOS, ideal gas (hydro_ve/eos.hpp:191-197) -> prho, c, and rho, p when non-null */
int sphgb_compute_eos(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeIadDivvCurlv (hydro_ve/iad_divv_curlv.hpp:93-98) -> c11..c33, divv, curlv (if
 * non-null), dV11..dV33 (if non-null) */
int sphgb_compute_iad_divv_curlv(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeAVswitches (hydro_ve/av_switches.hpp:81-86) -> alpha (in/out), dt = params.minDt */
int sphgb_compute_av_switches(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::computeMomentumEnergy<avClean> (hydro_ve/momentum_energy.hpp:107-115) -> ax ay az du;
 * group_dt: optional device float per 32-particle group (reference groupDt); minDtCourant as
 * above */
int sphgb_compute_momentum_energy(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last,
                                  int32_t av_clean, float* group_dt, double* minDtCourant);

/* ---- whole sweep: sync + neighbours + the pair passes of one propagator step
 *      (main/src/propagator/std_hydro.hpp:124-168, ve_hydro.hpp:130-204) ----
 * Positions, velocities and h cannot change between the passes of one call, so the FP64 VE sweep
 * (default mode) forms each owned pair's geometry and kernel values once, in the xmass pass, and
 * the later passes read them: a context-owned buffer of up to 80 bytes per owned pair (8M
 * particles: 35 GB), taken only when it fits in half of the free device memory, kept between
 * calls, given back when larger neighbour lists need the space.  The pass entry points above form
 * the geometry in every call. */
int sphgb_sweep(sphgb_ctx* ctx, sphgb_particles* p, sphgb_box* box, int32_t variant, int32_t av_clean,
                double* minDtCourant);
/* same chain without the domain sync (keys, sort, tree reused): the frozen-tree sweep */
int sphgb_sweep_passes(sphgb_ctx* ctx, sphgb_particles* p, int32_t variant, int32_t av_clean,
                       double* minDtCourant);

/* ---- adjoint ----
 * No reference counterpart (the reference has no gradients).  Reverse mode of the std chain
 * density -> EOS -> IAD -> momentum-energy, for the state left by the last forward passes on the
 * frozen neighbour lists of the last search (over all particles, first = 0, last = n), in the
 * form of those passes: FP64, or mixed (FP32 pair arithmetic on the forward's grid-form coordinate
 * differences, FP32 sums, FP64 gradients out; seeds rho, a in the field type; deterministic = 1 is
 * refused for the mixed form).
 * Seeds are dL/d(output) per particle (device, double; NULL = zero); outputs are dL/d(input)
 * (device, double).  The Courant time step is not differentiated. */
typedef struct {
    const void *rho, *ax, *ay, *az;   /* dL/drho, dL/da */
    const double* du;                 /* dL/ddu */
} sphgb_seeds;

typedef struct {
    double *x, *y, *z;                /* dL/dx */
    double *vx, *vy, *vz;             /* dL/dv */
    double *h, *u;                    /* dL/dh, dL/du */
} sphgb_grads;

/* deterministic = 0: every pair is differentiated once and the neighbour's partials are added
 * with FP64 atomics (fastest; sums in arrival order).  deterministic = 1: every pair is
 * differentiated from both ends, the neighbour end walking an incoming-list CSR built once per
 * list set, and each particle sums its own terms in a fixed order (bit-reproducible); that CSR
 * takes fewer than 2^32 list entries (SPHGB_ERR_TOO_LARGE otherwise). */
int sphgb_adjoint_std(sphgb_ctx* ctx, sphgb_particles* p, const sphgb_seeds* seeds, sphgb_grads* grads,
                      int32_t deterministic);

/* Reverse mode of the VE chain xmass -> kx/gradh -> EOS -> IAD + divv/curlv (+dV) -> AV switches ->
 * momentum-energy<av_clean> (ve_hydro.hpp:130-204), for the state left by the last forward VE
 * passes on the frozen lists of the last search (first = 0, last = n), FP64 form.  alpha_prev is
 * alpha before the AV switch of that forward (the switch updates p->alpha in place); the time step
 * of the switch is params.minDt.  Seeds: rho (= kx m / xm), a, du; outputs as sphgb_adjoint_std.
 * The AV switch and the Atwood weights are differentiated piecewise, on the branch the forward
 * took; the Courant time step is not differentiated.  deterministic as sphgb_adjoint_std. */
int sphgb_adjoint_ve(sphgb_ctx* ctx, sphgb_particles* p, const double* alpha_prev, int32_t av_clean,
                     const sphgb_seeds* seeds, sphgb_grads* grads, int32_t deterministic);

/* ---- statistics and timing ---- */
int sphgb_get_stats(sphgb_ctx* ctx, sphgb_stats* stats);
/* milliseconds of the last call of each stage, measured with CUDA events on the context
 * stream: [0] sync [1] neighbours [2..7] pair passes in call order of the last sweep */
int sphgb_get_timings(sphgb_ctx* ctx, float* ms, int32_t count);
/* number of kernels this library launched since the context was created */
int sphgb_kernel_launches(sphgb_ctx* ctx, int64_t* launches);
/* device-wide FMA throughput (FLOP/s, FMA = 2) of the FP64 (fp64 != 0) or FP32 pipe, measured
 * with a dependent-chain probe kernel; the roofline denominator of the pair passes (no
 * reference counterpart: the reference records no performance figures) */
int sphgb_measure_fma_peak(sphgb_ctx* ctx, int32_t fp64, double* flops_per_s);

/* ---- time integration and reductions (one time step for all particles, no rungs) ---- */

/* Timestep state of sphexa::ParticlesData used by sph::computeTimestep (ts_global.hpp:97-113). */
typedef struct {
    double minDt, minDt_m1, ttot;   /* in/out: current and previous step, elapsed time */
    double minDtCourant;            /* in: Courant limit from the momentum-energy pass */
    double minDtRho;                /* in: divv limit (sphgb_rho_timestep), INFINITY if unused */
    double maxDtIncrease;           /* in: growth limit, 1.1 in the reference (particles_data.hpp:141) */
    double g, etaAcc, eps;          /* in: acceleration limit when g != 0 (ts_global.hpp:36-57);
                                       reference defaults etaAcc 0.2, eps 0.005 (particles_data.hpp:112-114) */
} sphgb_timestep;

/* sph::computePositions (sph/include/sph/positions.hpp:180-200; GPU computePositionsKernel,
 * positions_gpu.cu:118-165) on [first, last) with dt = ts->minDt and dt_m1 = ts->minDt_m1: Press
 * position update with the periodic put-in-box, velocities at n+1, X_n+1 - X_n into x_m1 y_m1 z_m1,
 * Adams-Bashforth update of u with du_m1 <- du; particles at rest within 2h of a fixed boundary do
 * not move.  x_m1 y_m1 z_m1 du_m1 have the precision's hydro type (double or float). */
int sphgb_compute_positions(sphgb_ctx* ctx, sphgb_particles* p, const sphgb_box* box, void* x_m1, void* y_m1,
                            void* z_m1, void* du_m1, const sphgb_timestep* ts, int64_t first, int64_t last);
/* sph::updateSmoothingLength (sph/include/sph/update_h.hpp:26-45, updateH kernels.hpp:26-32):
 * h <- h/2 (1 + 1023 ng0 / nc)^(1/10) with nc the neighbour counts of the last search (p->nc) */
int sphgb_update_smoothing_length(sphgb_ctx* ctx, sphgb_particles* p, int64_t first, int64_t last);
/* sph::rhoTimestep (ts_global.hpp:72-95): Krho / |max divv| over [first, last); the reference's
 * Krho is 0.06 (particles_data.hpp:107) */
int sphgb_rho_timestep(sphgb_ctx* ctx, const sphgb_particles* p, int64_t first, int64_t last, double Krho,
                       double* dt);
/* sph::accelerationTimestep (ts_global.hpp:36-57): etaAcc sqrt(eps / sqrt(max |a|^2)) */
int sphgb_acceleration_timestep(sphgb_ctx* ctx, const sphgb_particles* p, int64_t first, int64_t last,
                                double etaAcc, double eps, double* dt);
/* sph::computeTimestep at one rank (ts_global.hpp:97-113): min of the acceleration limit (g != 0),
 * minDtCourant, minDtRho and maxDtIncrease * minDt; updates ttot, minDt_m1, minDt */
int sphgb_compute_timestep(sphgb_ctx* ctx, const sphgb_particles* p, int64_t first, int64_t last,
                           sphgb_timestep* ts);
/* sphexa::localConservedQuantities (main/src/observables/conserved_quantities.hpp:49-113; GPU
 * conservedQuantitiesGpu, conserved_gpu.cu:71-95) with u: out = {eKin, eInt, px, py, pz, Lx, Ly, Lz},
 * FP64 sums in a fixed order (run-to-run identical) */
int sphgb_conserved_quantities(sphgb_ctx* ctx, const sphgb_particles* p, int64_t first, int64_t last,
                               double out[8]);

/* ---- allocation-free entry point ----
 * No counterpart in the reference.  For callers that must not let a library call cudaMalloc or
 * cudaFree (their device memory is owned by their own pool allocator, or they cannot afford the
 * implicit device synchronisation of allocation inside a time-step loop): fits the open box
 * dimensions to the particle extrema like the first sphgb_domain_sync of a simulation (it keeps no
 * previous box, so the limitBoxShrinking of domain mode 1 does not apply) and writes the Hilbert
 * key of every particle, in input order, into `keys` (device, n entries).  x, y, z are device
 * pointers; `box` is a host struct, updated in place.  Needs no context and allocates nothing: its
 * reduction scratch is a fixed 3 MiB device array inside the library (held by every GPU that loads
 * it until the process exits), which caps n at 268,435,456; larger n returns SPHGB_ERR_TOO_LARGE.
 * The first call on a device looks up that array's device address with cudaGetSymbolAddress; the
 * address is kept for the life of the process, so do not call this entry point on a device after
 * cudaDeviceReset of that device.  Every call shares the array: calls that overlap on the GPU, on
 * one device, race.  Runs on `stream` (0 = legacy default) and returns after synchronising it (the
 * open-box path also reads the extrema back to the host), so a call cannot be part of a stream
 * capture (CUDA graph). */
int sphgb_sfc_keys_noalloc(const double* x, const double* y, const double* z, int64_t n, sphgb_box* box,
                           uint64_t* keys, void* stream);


#ifdef __cplusplus
}
#endif

#endif /* SPHGB_H */
