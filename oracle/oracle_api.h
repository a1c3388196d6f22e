/*
 * Oracle C API — TEST INFRASTRUCTURE ONLY.
 *
 * Two libraries implement this header with identical signatures:
 *   - oracle/liboracle.so : a CPU restatement (oracle/port/oracle.cpp) of OMPL's algorithms for the
 *                           sampling / validity / discrete-motion / nearest-neighbour path. It
 *                           builds anywhere g++ runs and is the checker on the GPU machine.
 *   - oracle/_ref/libompl_ref.so : OMPL's own sources compiled unmodified (oracle/ref/Makefile),
 *                           available only where the OMPL source tree is present. It pins the
 *                           restatement and generates the golden fixtures in tests/golden/.
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline leg may load either library.
 * The product library (libgbompl.so) never links or calls anything here.
 *
 * Conventions: states are row-major AoS (n rows of `dim` doubles), as OMPL stores a
 * RealVectorStateSpace::StateType::values array per state. All arithmetic is FP64 and the
 * libraries are compiled with -ffp-contract=off, so no multiply-add is fused.
 */
#ifndef GBOMPL_ORACLE_API_H
#define GBOMPL_ORACLE_API_H

#ifdef __cplusplus
extern "C" {
#endif

/* State-space kinds. */
enum {
    ORA_SPACE_REAL_VECTOR = 0,      /* ompl::base::RealVectorStateSpace */
    ORA_SPACE_SO2 = 1,              /* ompl::base::SO2StateSpace (dim must be 1) */
    ORA_SPACE_KINEMATIC_CHAIN = 2,  /* KinematicChainSpace of demos/KinematicChain.h */
    ORA_SPACE_WRAP_L2 = 3           /* RealVector(dim) on [-pi,pi]^dim, L2 over wrapped joint differences */
};

/* Validity-checker kinds. */
enum {
    ORA_CHECK_ALL_VALID = 0,        /* ompl::base::AllValidStateValidityChecker */
    ORA_CHECK_CIRCLES = 1,          /* point robot vs circles: obstacles are (x, y, r) rows */
    ORA_CHECK_CHAIN_SEGMENTS = 2,   /* KinematicChainValidityChecker: obstacles are (x0, y0, x1, y1) rows */
    ORA_CHECK_DH_SPHERES = 3,       /* serial DH arm covered by spheres vs world spheres (x, y, z, r) rows */
    ORA_CHECK_DH_BOXES = 4          /* the same arm vs axis-aligned boxes (cx, cy, cz, hx, hy, hz) rows */
};

/* Nearest-neighbour structures (the reference library honours all; the restatement only EXACT). */
enum {
    ORA_NN_EXACT = 0,               /* linear scan ordered by (distance, insertion index) */
    ORA_NN_REF_LINEAR = 1,          /* ompl::NearestNeighborsLinear (ties unspecified) */
    ORA_NN_REF_GNAT = 2,            /* ompl::NearestNeighborsGNAT */
    ORA_NN_REF_GNAT_NTS = 3,        /* ompl::NearestNeighborsGNATNoThreadSafety */
    ORA_NN_REF_SQRT_APPROX = 4      /* ompl::NearestNeighborsSqrtApprox */
};

typedef struct {
    int kind;
    int dim;
    const double *low;      /* REAL_VECTOR bounds (dim entries); ignored by the other kinds */
    const double *high;
    double link_length;     /* KINEMATIC_CHAIN only */
    double lvs_fraction;    /* StateSpace::setLongestValidSegmentFraction */
    unsigned factor;        /* StateSpace::setValidSegmentCountFactor */
} ora_space;

typedef struct {
    int kind;
    const double *obstacles;    /* row-major obstacle records, layout per kind above */
    long n_obstacles;
    const double *dh;           /* DH_SPHERES: n_joints rows of (a, d, alpha_code) with alpha_code in {0,+1,-1}
                                   meaning alpha = 0, +pi/2, -pi/2 */
    int n_joints;
    int spheres_per_link;
    double sphere_radius;
} ora_checker;

/* Worker threads used by the batch loops below (>= 1). Returns the previous value. */
int ora_set_threads(int n);

/* StateSpace::getMaximumExtent and getLongestValidSegmentLength after StateSpace::setup. */
double ora_space_extent(const ora_space *s);
double ora_space_lvs(const ora_space *s);

/* Per-row distance(a_i, b_i), interpolate(a_i, b_i, t_i) and validSegmentCount(a_i, b_i). */
void ora_distance(const ora_space *s, const double *a, const double *b, long n, double *out);
void ora_interpolate(const ora_space *s, const double *a, const double *b, const double *t, long n, double *out);
void ora_valid_segment_count(const ora_space *s, const double *a, const double *b, long n, unsigned *out);
void ora_enforce_bounds(const ora_space *s, double *states, long n);

/* The space's default state sampler, RNG seeded with setLocalSeed(seed): n consecutive draws. */
void ora_sample_uniform(const ora_space *s, unsigned seed, long n, double *out);
/* sampleUniformNear(out_i, near_i, distance) for i = 0..n-1 from one sampler. */
void ora_sample_uniform_near(const ora_space *s, unsigned seed, const double *near, double distance, long n,
                             double *out);
/* One sampler (RNG seeded with setLocalSeed(seed)) running a script of calls: call k draws counts[k]
 * states with sampleUniform (kinds[k] = 0) or with sampleGaussian around the next counts[k] rows of
 * mean, standard deviation stddev (kinds[k] = 1); out receives every drawn row in order.
 * log_mode (restatement only; the reference build takes 0): 0 = std::normal_distribution, as OMPL;
 * 1 = the same polar method with the log rounded to nearest (ora_log_rn). */
void ora_sample_script(const ora_space *s, unsigned seed, const int *kinds, const long *counts, int nops,
                       const double *mean, double stddev, int log_mode, double *out);
/* Natural log rounded to nearest (double-double evaluation) of positive normal doubles. */
void ora_log_rn(const double *x, long n, double *out);
/* Raw RNG draws: uniform01 (kind 0) or uniformReal(lo, hi) (kind 1), n values from RNG(seed). */
void ora_rng_uniform(unsigned seed, int kind, double lo, double hi, long n, double *out);

/* StateValidityChecker::isValid for each row: out[i] = 1 valid, 0 invalid. */
void ora_is_valid(const ora_space *s, const ora_checker *c, const double *states, long n, unsigned char *out);

/* DiscreteMotionValidator on each edge (s1_i, s2_i):
 *   ok[i]       = checkMotion(s1, s2, lastValid)       (ordered variant)
 *   ok_bisect[i]= checkMotion(s1, s2)                  (bisection variant)          [nullable]
 *   last_t[i]   = lastValid.second, or NaN when the motion is valid                  [nullable]
 *   last_state  = lastValid.first rows (dim doubles), NaN rows when valid            [nullable]
 *   nd[i]       = validSegmentCount(s1, s2)                                          [nullable]
 *   first_j[i]  = index of the first invalid checked state in the ordered variant:
 *                 1..nd-1 for interpolated states, nd for s2 itself, -1 when valid   [nullable] */
void ora_check_motion(const ora_space *s, const ora_checker *c, const double *s1, const double *s2, long n,
                      unsigned char *ok, unsigned char *ok_bisect, double *last_t, double *last_state, int *nd,
                      int *first_j);

/* SpaceInformation::checkMotion(states, count, firstInvalidStateIndex) over rows [0, count):
 * returns 1 when all are valid; otherwise 0 and *first_invalid set. Bisection variant in *ok_bisect. */
int ora_check_motion_states(const ora_space *s, const ora_checker *c, const double *states, long count,
                            long *first_invalid, int *ok_bisect);

/* SpaceInformation::getMotionStates(s1, s2, states, count, endpoints, alloc=true): returns rows written. */
long ora_get_motion_states(const ora_space *s, const double *s1, const double *s2, unsigned count, int endpoints,
                           double *out);

/* nearestK over `pts` (insertion order = row index) for each query row. idx/dist are nq x k, padded
 * with -1 / +inf when fewer than k points exist. distance is evaluated as distance(point, query). */
void ora_knn(const ora_space *s, int algo, const double *pts, long npts, const double *q, long nq, int k,
             long *idx, double *dist);

/* NearestNeighborsSqrtApprox::nearest (NearestNeighborsSqrtApprox.h:91-115) for nq queries made one after
 * another on a fresh structure holding pts (added in one call), after removing the rows remove[0..nrem)
 * one at a time: idx[i] = the row returned for query i, dist[i] = its distance to the query. Returns the
 * structure's offset after the last query. */
unsigned long ora_nn_sqrt_approx(const ora_space *s, const double *pts, long npts, const long *remove, long nrem,
                                 const double *q, long nq, long *idx, double *dist);

/* PRM-order prefix nearestK: query i sees only points with row index < limit[i]. */
void ora_knn_prefix(const ora_space *s, const double *pts, long npts, const double *q, const long *limit, long nq,
                    int k, long *idx, double *dist);

/* nearestR (distance <= r): counts[i] per query; when idx/dist are non-null they receive the CSR
 * concatenation of the sorted results (capacity `cap` entries). Returns the total count. */
long ora_radius(const ora_space *s, int algo, const double *pts, long npts, const double *q, long nq, double r,
                long *counts, long *idx, double *dist, long cap);

#ifdef __cplusplus
}
#endif
#endif
