/* Oracle interface: ONE call runs the single-rank SPH hydro sweep on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Two implementations export this interface:
 *   - oracle/sph_oracle.cpp   my own C++/OpenMP restatement of the reference algorithm
 *                             (built into oracle/liboracle.so; travels to every machine);
 *   - oracle/ref/ref_driver.cpp  a thin driver that calls the reference's own headers
 *                             (built into oracle/_ref/ only where the reference sources exist).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load either.
 *
 * Chain (reference call stack C): makeGlobalBox -> computeSfcKeys -> stable sort_by_key
 * -> computeOctree(keys, bucket) -> updateInternalTree -> nodeFpCenters -> findNeighborsSph
 * -> {std: computeDensity, computeEOS_HydroStd, computeIAD, computeMomentumEnergySTD}
 *  | {ve:  computeXMass, computeVeDefGradh, computeEOS, computeIadDivvCurlv,
 *          computeAVswitches, computeMomentumEnergy<avClean>}.
 * All per-particle outputs are in SFC (sorted) order.
 */
#ifndef SPHGB_ORACLE_API_H
#define SPHGB_ORACLE_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* per-particle field slots of oracle_out.f (and of oracle_in.f for inputs) */
enum oracle_field {
    OF_X = 0, OF_Y, OF_Z, OF_H, OF_M, OF_U, OF_VX, OF_VY, OF_VZ, OF_ALPHA,
    OF_RHO, OF_P, OF_C, OF_C11, OF_C12, OF_C13, OF_C22, OF_C23, OF_C33,
    OF_AX, OF_AY, OF_AZ, OF_DU, OF_XM, OF_KX, OF_GRADH, OF_PRHO, OF_DIVV, OF_CURLV,
    OF_DV11, OF_DV12, OF_DV13, OF_DV22, OF_DV23, OF_DV33,
    OF_NFIELDS
};

enum oracle_stage {
    OS_KEYS = 1,   /* box, keys, stable sort, gather */
    OS_TREE = 2,   /* cornerstone leaves, internal octree, node centers */
    OS_NBR  = 4,   /* neighbour search with h iteration */
    OS_HYDRO = 8   /* pair passes of the selected variant */
};

typedef struct {
    int64_t n;
    const double* f[OF_NFIELDS]; /* inputs, unsorted: x y z h m u vx vy vz alpha used */
    double box[6];               /* xmin xmax ymin ymax zmin zmax */
    uint8_t bc[3];               /* 0 open, 1 periodic */
    uint8_t fit_box;             /* 1: open dimensions take the particle extrema */
    uint32_t ng0, ngmax, bucket;
    double gamma, Kcour, minDt, alphamin, alphamax, decay, sincIndex;
    int32_t variant;             /* 0 std, 1 ve */
    int32_t avclean;
    int32_t stages;              /* oracle_stage bitmask */
    int32_t nthreads;            /* 0: OpenMP default */
} oracle_in;

typedef struct {
    /* capacities given by the caller; NULL pointers are skipped */
    uint64_t* keys;              /* [n] sorted keys */
    uint32_t* order;             /* [n] original index of each sorted particle */
    int64_t leaves_cap;          /* capacity of leaves (>= num_leaves + 1) */
    uint64_t* leaves;            /* cornerstone leaf keys */
    uint32_t* counts;            /* particles per leaf */
    int64_t nodes_cap;
    uint64_t* prefixes;          /* octree node keys, placeholder-bit format, level-major */
    int32_t* child_offsets;
    int32_t* internal_to_leaf;
    uint32_t* nc;                /* [n] neighbour count incl. self */
    uint32_t* nbr;               /* [n * ngmax] neighbour indices, reference layout i*ngmax+k */
    double* f[OF_NFIELDS];       /* [n] outputs, sorted order */
    /* scalar outputs */
    double box[6];
    int64_t num_leaves, num_nodes, num_internal;
    int32_t level_range[23];
    int64_t h_iter_fails;
    double minDtCourant;
    double t_keys, t_tree, t_nbr, t_hydro;   /* wall seconds per stage */
    int32_t threads_used;
    double* centers;             /* [3 * nodes_cap] geometric node centers (nodeFpCenters), x y z per node */
    double* sizes;               /* [3 * nodes_cap] geometric node half sizes */
} oracle_out;

int oracle_sweep(const oracle_in* in, oracle_out* out);

/* One j-loop for particle 0 over an explicit neighbour list, as the reference's known-answer
 * tests call them (sph/test/std.cpp:98-127, sph/test/ve.cpp:112-233). */
enum oracle_jloop_kind {
    OJ_XMASS = 0,   /* out: xm */
    OJ_GRADH,       /* out: kx, gradh */
    OJ_IAD_STD,     /* out: c11 c12 c13 c22 c23 c33 (volume m/rho) */
    OJ_IAD_VE,      /* out: c11 .. c33 (volume xm/kx) */
    OJ_DIVV,        /* out: divv curlv dV11 dV12 dV13 dV22 dV23 dV33 */
    OJ_AV,          /* out: alpha */
    OJ_ME_STD,      /* out: ax ay az du maxvsignal */
    OJ_ME_VE        /* out: ax ay az du maxvsignal (avclean selects the AV cleaning) */
};

typedef struct {
    int64_t n;
    const double* f[OF_NFIELDS];   /* per-particle inputs by slot; NULL reads as zeros */
    const uint32_t* neighbors;     /* neighbour list of particle 0 */
    uint32_t count;
    double K;                      /* kernel normalisation to use */
    double box[6];
    uint8_t bc[3];
    double sincIndex;
    double dt, alphamin, alphamax, decay;
    int32_t loop;                  /* oracle_jloop_kind */
    int32_t avclean;
} oracle_jloop_in;

int oracle_jloop(const oracle_jloop_in* in, double* out);
/* kernel normalisation constant and tables for a sinc^n kernel, for table-level checks */
double oracle_kernel_K(double sincIndex);
void oracle_tables(double sincIndex, double* wh, double* whd); /* 20000 each */

/* One integration step for all particles (FP64 fields), the semantics of the reference GPU path
 * (computePositionsKernel, sph/include/sph/positions_gpu.cu:118-165): Press position update with
 * put-in-box, velocities at n+1, X_n+1 - X_n into xm1, Adams-Bashforth u update with dum1 <- du;
 * particles at rest within 2h of a fixed boundary (bc 2) are left untouched. */
int oracle_positions(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                     const double* ax, const double* ay, const double* az, double* xm1, double* ym1, double* zm1,
                     double* u, const double* du, double* dum1, const double* h, double dt, double dt_m1,
                     const double box[6], const uint8_t bc[3]);
/* updateH (sph/include/sph/kernels.hpp:26-32) for every particle */
int oracle_update_h(int64_t n, uint32_t ng0, const uint32_t* nc, double* h);
/* localConservedQuantities with u (main/src/observables/conserved_quantities.hpp:49-113):
 * out = {eKin, eInt, px, py, pz, Lx, Ly, Lz}, sequential sums in index order */
int oracle_conserved(int64_t n, const double* x, const double* y, const double* z, const double* vx,
                     const double* vy, const double* vz, const double* m, const double* u, double out[8]);

#ifdef __cplusplus
}
#endif

#endif
