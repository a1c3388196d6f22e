/*
 * gbompl — GB300 (sm_103a) implementation of OMPL's data-parallel inner loop behind a C ABI:
 * state sampling, state validity, discrete motion checking and nearest-neighbour queries.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns a gbo_status and never
 * throws. Device-pointer calls are asynchronous on the given stream (NULL = legacy default stream);
 * `*_host` calls take host arrays and return when results are on the host.
 *
 * State layout. A batch of n states of dimension `dim` is passed as (ptr, n, ld, layout):
 *   GBO_LAYOUT_SOA: value (i, d) at ptr[d * ld + i], ld >= n (coalesced; the native layout);
 *   GBO_LAYOUT_AOS: value (i, d) at ptr[i * ld + d], ld >= dim (OMPL's per-state double arrays).
 *
 * Reference interfaces replaced (paths inside the OMPL source tree):
 *   StateSampler::sampleUniform / sampleUniformNear        src/ompl/base/StateSampler.h:79-88
 *     with RealVectorStateSampler / SO2StateSampler        src/ompl/base/spaces/src/RealVectorStateSpace.cpp:45-65,
 *                                                           src/ompl/base/spaces/src/SO2StateSpace.cpp:46-56
 *   StateValidityChecker::isValid                         src/ompl/base/StateValidityChecker.h:111
 *   MotionValidator::checkMotion (both overloads), with    src/ompl/base/MotionValidator.h:83,99
 *     DiscreteMotionValidator semantics                    src/ompl/base/src/DiscreteMotionValidator.cpp:48-145
 *   StateSpace::validSegmentCount / distance / interpolate src/ompl/base/src/StateSpace.cpp:851-854
 *   SpaceInformation::checkMotion(states, count, first)    src/ompl/base/src/SpaceInformation.cpp:288-341
 *   NearestNeighbors<T>::add/remove/nearestK/nearestR/size/clear
 *                                                          src/ompl/datastructures/NearestNeighbors.h:58-110
 */
#ifndef GBOMPL_H
#define GBOMPL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gbo_status;
enum {
    GBO_OK = 0,
    GBO_ERR_INVALID_ARGUMENT = 1, /* bad handle, size, kind or pointer (OMPL throws ompl::Exception here) */
    GBO_ERR_CUDA = 2,             /* a CUDA runtime call failed; gbo_last_error() has the message */
    GBO_ERR_NO_DEVICE = 3,        /* no CUDA device, or not an sm_103 device */
    GBO_ERR_OUT_OF_MEMORY = 4,    /* device or pinned allocation failed / admission refused */
    GBO_ERR_TIMEOUT = 5,          /* a bounded device-side wait ran out (kernel returned early) */
    GBO_ERR_UNSUPPORTED = 6       /* combination not implemented (e.g. dim above 16) */
};

typedef struct gbo_space gbo_space;       /* a state space: metric, interpolation, bounds, segment length */
typedef struct gbo_checker gbo_checker;   /* a validity checker bound to a space and a device-resident world */
typedef struct gbo_sampler gbo_sampler;   /* a state sampler with its own mt19937 stream */
typedef struct gbo_nn gbo_nn;             /* a device-resident nearest-neighbour index */
typedef void *gbo_stream;                 /* a cudaStream_t */

enum { GBO_LAYOUT_SOA = 0, GBO_LAYOUT_AOS = 1 };

enum {
    GBO_SPACE_REAL_VECTOR = 0,     /* RealVectorStateSpace: L2, linear interpolation, box bounds */
    GBO_SPACE_SO2 = 1,             /* SO2StateSpace (dim 1) */
    GBO_SPACE_KINEMATIC_CHAIN = 2, /* KinematicChainSpace of demos/KinematicChain.h (param = link length) */
    GBO_SPACE_WRAP_L2 = 3          /* joint space on [-pi,pi]^dim, L2 over wrapped differences */
};

enum {
    GBO_CHECK_ALL_VALID = 0,      /* AllValidStateValidityChecker */
    GBO_CHECK_CIRCLES = 1,        /* point robot vs circles; world rows (x, y, r) */
    GBO_CHECK_CHAIN_SEGMENTS = 2, /* KinematicChainValidityChecker; world rows (x0, y0, x1, y1) */
    GBO_CHECK_DH_SPHERES = 3,     /* DH serial arm covered by spheres vs world spheres (x, y, z, r) */
    GBO_CHECK_DH_BOXES = 4        /* the same arm vs axis-aligned boxes (cx, cy, cz, hx, hy, hz): centre and
                                     half extents; no reference counterpart (the reference has no
                                     collision checker of its own), definition in oracle/dh_arm.h */
};

/* Arithmetic of validity / motion / kNN evaluation. */
enum {
    GBO_PRECISION_FP64 = 0,        /* FP64 throughout, reference operation order (the plain form) */
    GBO_PRECISION_FP32_GUARDED = 1 /* FP32 bulk; anything within the guard band re-evaluated in FP64 */
};

/* Motion-batch schedules. */
enum {
    GBO_SCHEDULE_PLAIN = 0, /* one launch, one warp per edge, 32 steps per ballot, FP64 (drop-in) */
    GBO_SCHEDULE_TILE = 1,  /* persistent: 32 edges per warp, lanes re-spread over live edges */
    GBO_SCHEDULE_WARP = 2,  /* persistent: one warp per edge from the work queue */
    GBO_SCHEDULE_AUTO = 3   /* autotuned between TILE and WARP (cached per checker) */
};

/* ---- errors / device ---- */
const char *gbo_status_string(gbo_status s);
const char *gbo_last_error(void); /* message of the last failure on this thread ("" if none) */
gbo_status gbo_device_check(int *sm_count, int *cc_major, int *cc_minor);

/* ---- state spaces ---- (StateSpace::setup, getLongestValidSegmentLength, validSegmentCount)
 * low/high: dim bounds (REAL_VECTOR only; may be NULL otherwise). lvs and factor are the values the
 * OMPL space reports (getLongestValidSegmentLength(), getValidSegmentCountFactor()); pass lvs <= 0 to
 * have them computed as maximumExtent * lvs_fraction like StateSpace::setup. */
gbo_status gbo_space_create(int kind, int dim, const double *low, const double *high, double param, double lvs,
                            double lvs_fraction, unsigned factor, gbo_space **out);
gbo_status gbo_space_destroy(gbo_space *s);
gbo_status gbo_space_info(const gbo_space *s, double *max_extent, double *lvs);
/* distance(a_i, b_i), interpolate(a_i, b_i, t_i), validSegmentCount(a_i, b_i) over batches (device). */
gbo_status gbo_space_distance(const gbo_space *s, const double *a, const double *b, int64_t n, int64_t ld, int layout,
                              double *out, gbo_stream stream);
gbo_status gbo_space_interpolate(const gbo_space *s, const double *a, const double *b, const double *t, int64_t n,
                                 int64_t ld, int layout, double *out, gbo_stream stream);
/* SpaceInformation::getMotionStates(s1, s2, states, count, endpoints, alloc = true)
 * (src/ompl/base/src/SpaceInformation.cpp:215-286) over a batch of edges: edge i yields
 * m = count + 2 states with endpoints (s1, interpolate(s1, s2, j / (count + 1)) for j = 1..count, s2)
 * or m = count without, as rows i*m .. i*m + m - 1 of out (n*m rows, out_ld, same layout). */
gbo_status gbo_get_motion_states(const gbo_space *s, const double *s1, const double *s2, int64_t n, int64_t ld,
                                 int layout, unsigned count, int endpoints, double *out, int64_t out_ld,
                                 gbo_stream stream);

/* ---- validity checkers ----
 * world: n_world rows of 3 (circles), 4 (segments, spheres) or 6 (boxes) doubles, host memory, copied to
 * the device.
 * dh: n_joints rows (a, d, alpha_code), alpha_code in {0, +1, -1} = alpha 0, +pi/2, -pi/2 (DH_SPHERES). */
gbo_status gbo_checker_create(const gbo_space *space, int kind, const double *world, int64_t n_world,
                              const double *dh, int n_joints, int spheres_per_link, double sphere_radius,
                              gbo_checker **out);
gbo_status gbo_checker_destroy(gbo_checker *c);
gbo_status gbo_checker_set_precision(gbo_checker *c, int precision);
/* Re-check statistics of the last FP32_GUARDED call: states evaluated, states re-checked in FP64. */
gbo_status gbo_checker_stats(const gbo_checker *c, uint64_t *evaluated, uint64_t *rechecked);
/* The same counters of the last call plus its one-ulp hazards: FP64 decisions (segment-test or sphere
 * comparisons) so close to their thresholds that a one-ulp change of a sine or cosine of the forward
 * kinematics could reverse them. The FP64 forms use correctly rounded sin/cos; the reference calls the
 * C library's, which differs by one ulp on a small fraction of arguments, so a call with no hazard
 * decided every FP64 comparison as the reference does. No reference counterpart (diagnostic). */
gbo_status gbo_checker_counters(const gbo_checker *c, uint64_t *evaluated, uint64_t *rechecked, uint64_t *hazards);

/* Precision statistics of the FP32 form on a batch of states (measurement call; synchronous; allocates
 * a small device buffer): states, flips = states whose FP32 verdict taken at face value (the reference's
 * comparisons on the FP32 values, no guard band) differs from the FP64 verdict, ambiguous = states the
 * guarded FP32 form hands to the FP64 re-check, max_abs_err = largest |FP32 - FP64| of the compared
 * quantities (chain: segment-test denominators and numerators; DH arm: d^2 - (rs + ro)^2 of the listed
 * sphere pairs). GBO_ERR_UNSUPPORTED for checkers without an FP32 form (circles, all-valid).
 * No reference counterpart (diagnostic). */
typedef struct
{
    uint64_t states;
    uint64_t flips;
    uint64_t ambiguous;
    double max_abs_err;
} gbo_precision_stats;
gbo_status gbo_checker_precision_stats(gbo_checker *c, const double *states, int64_t n, int64_t ld, int layout,
                                       gbo_precision_stats *out, gbo_stream stream);

/* StateValidityChecker::isValid over a batch: out[i] = 1 valid, 0 invalid. */
gbo_status gbo_is_valid(gbo_checker *c, const double *states, int64_t n, int64_t ld, int layout, uint8_t *out,
                        gbo_stream stream);

/* DiscreteMotionValidator::checkMotion over a batch of edges (s1_i -> s2_i):
 *   ok[i]      1 when the motion is valid (both overloads agree on this);
 *   first_j[i] ordered-variant index of the first invalid checked state: 1..nd-1 interpolated,
 *              nd for s2 itself, -1 when valid [nullable];
 *   nd[i]      validSegmentCount(s1, s2) [nullable].
 * lastValid.second = (first_j - 1) / nd (FP64 division, as DiscreteMotionValidator.cpp:66,79) and
 * lastValid.first = interpolate(s1, s2, lastValid.second) are produced by gbo_last_valid. */
gbo_status gbo_check_motion(gbo_checker *c, const double *s1, const double *s2, int64_t n, int64_t ld, int layout,
                            int schedule, uint8_t *ok, int32_t *first_j, int32_t *nd, gbo_stream stream);
gbo_status gbo_last_valid(const gbo_space *s, const double *s1, const double *s2, const int32_t *first_j,
                          const int32_t *nd, int64_t n, int64_t ld, int layout, double *last_t, double *last_state,
                          gbo_stream stream);
/* SpaceInformation::checkMotion(states, count, firstInvalidStateIndex): one ordered chain of states. */
gbo_status gbo_check_motion_states(gbo_checker *c, const double *states, int64_t count, int64_t ld, int layout,
                                   uint8_t *ok, int64_t *first_invalid, gbo_stream stream);

/* Host-memory drop-ins (AoS rows like OMPL states); staging buffers are owned by the checker. */
gbo_status gbo_is_valid_host(gbo_checker *c, const double *states, int64_t n, uint8_t *out);
gbo_status gbo_check_motion_host(gbo_checker *c, const double *s1, const double *s2, int64_t n, uint8_t *ok,
                                 double *last_t, double *last_state);

/* ---- samplers ---- RNG seeded like RNG::setLocalSeed(seed); one sampler = one sequential stream. */
gbo_status gbo_sampler_create(const gbo_space *space, uint32_t local_seed, gbo_sampler **out);
gbo_status gbo_sampler_destroy(gbo_sampler *s);
gbo_status gbo_sample_uniform(gbo_sampler *s, int64_t n, double *out, int64_t ld, int layout, gbo_stream stream);
gbo_status gbo_sample_uniform_near(gbo_sampler *s, const double *near, double distance, int64_t n, int64_t ld,
                                   int layout, double *out, gbo_stream stream);
/* StateSampler::sampleGaussian (src/ompl/base/StateSampler.h:96-100; RealVectorStateSpace.cpp:67-82,
 * SO2StateSpace.cpp:58-62) for n states: row i of out drawn around row i of mean (same ld and layout)
 * with standard deviation stddev per coordinate, clamped to the bounds (wrapped for SO2). The values
 * come from RNG::gaussian (src/ompl/util/RandomNumbers.h:98-101, libstdc++'s polar method) and its
 * cached second value carries across calls of s, as OMPL's does; log is rounded to nearest, so a pair
 * whose log glibc rounds the other way differs in the last bits (the stream position never does).
 * Device arrays; returns when done (the host reads each chunk's accepted-candidate count). */
gbo_status gbo_sample_gaussian(gbo_sampler *s, const double *mean, double stddev, int64_t n, int64_t ld, int layout,
                               double *out, gbo_stream stream);
/* UniformValidStateSampler::sample (src/ompl/base/samplers/src/UniformValidStateSampler.cpp:46-57)
 * called n times: call i draws sampleUniform states from s until c reports one valid or `attempts`
 * were drawn (MAX_VALID_SAMPLE_ATTEMPTS = 100 in OMPL); row i of out = the state it ended on,
 * ok[i] = 1 when valid. The stream of s advances by exactly the draws the n calls make, as OMPL's
 * would. Device arrays; returns when done (the host decides how many states each round draws). */
gbo_status gbo_sample_valid(gbo_sampler *s, gbo_checker *c, int64_t n, unsigned attempts, double *out, int64_t ld,
                            int layout, uint8_t *ok, gbo_stream stream);

/* ---- nearest neighbours ---- (NearestNeighbors<T>; element key = insertion index) */
gbo_status gbo_nn_create(const gbo_space *space, int64_t capacity, gbo_nn **out);
gbo_status gbo_nn_destroy(gbo_nn *nn);
gbo_status gbo_nn_set_precision(gbo_nn *nn, int precision);
gbo_status gbo_nn_add(gbo_nn *nn, const double *states, int64_t n, int64_t ld, int layout, int64_t *first_key,
                      gbo_stream stream);
gbo_status gbo_nn_remove(gbo_nn *nn, const int64_t *keys, int64_t n, gbo_stream stream);
gbo_status gbo_nn_clear(gbo_nn *nn);
gbo_status gbo_nn_size(const gbo_nn *nn, int64_t *size);
/* nearestK: idx/dist are nq x k row-major, sorted by (distance, key); -1 / +inf padding when fewer
 * than k elements; 1 <= k <= 64 (the FP32-guarded form covers k <= 64 on RealVector / wrapped spaces
 * of dim <= 8 and k <= 20 on the chain space; larger k there runs the FP64 scan).
 * prefix (nullable): query i only sees keys < prefix[i] (PRM insertion order).
 * dist may be NULL. distance is evaluated as distance(element, query), like NearestNeighborsLinear. */
gbo_status gbo_nn_nearest_k(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, int k,
                            const int64_t *prefix, int64_t *idx, double *dist, gbo_stream stream);
/* nearestR (distance <= r): counts per query, then the CSR fill given the exclusive-scan offsets. */
gbo_status gbo_nn_nearest_r_count(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, double r,
                                  int64_t *counts, gbo_stream stream);
gbo_status gbo_nn_nearest_r_fill(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, double r,
                                 const int64_t *offsets, int64_t *idx, double *dist, gbo_stream stream);
gbo_status gbo_nn_stats(const gbo_nn *nn, uint64_t *queries, uint64_t *rechecked, uint64_t *fallbacks);
/* NearestNeighborsSqrtApprox::nearest (src/ompl/datastructures/NearestNeighborsSqrtApprox.h:91-115) for nq
 * queries made one after another: query i examines 1 + floor(sqrt(n)) of the n present elements, those
 * at positions (j * checks + offset_i) % n in insertion order, and returns the first strict minimum of the
 * FP64 distance (idx[i] = its key, dist[i] = the distance). *offset holds the structure's offset before
 * the first query and receives it after the last (0 for a new or cleared structure). An empty index
 * gives GBO_ERR_INVALID_ARGUMENT (OMPL throws). Queries on ld / layout; outputs are device arrays. */
gbo_status gbo_nn_nearest_sqrt_approx(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout,
                                      uint64_t *offset, int64_t *idx, double *dist, gbo_stream stream);
/* The same on host arrays (AoS rows; synchronous). */
gbo_status gbo_nn_nearest_sqrt_approx_host(gbo_nn *nn, const double *q, int64_t nq, uint64_t *offset, int64_t *idx,
                                           double *dist);

/* FP32 metric error of the last FP32_GUARDED nearestK call (no OMPL counterpart): the largest
 * |distance_fp32 - distance_fp64| over the candidates it re-checked in FP64, and the bound the guard band
 * assumes for it (the re-check band is twice that bound). */
gbo_status gbo_nn_error_stats(const gbo_nn *nn, float *max_abs_error, float *bound);

/* Bytes of element features and cell / chunk boxes that the last nearestK call's chain cell search read
 * (no OMPL counterpart; the algorithmic traffic of that search, for its roofline). 0 for other paths. */
gbo_status gbo_nn_search_bytes(const gbo_nn *nn, uint64_t *bytes);

/* nearestK exactly as gbo_nn_nearest_k, but the call allocates no device memory (no counterpart in
 * OMPL). For callers that cannot allocate once set up: work captured into CUDA graphs, real-time
 * planning loops, processes whose GPU memory belongs to another allocator's pool. Scratch comes from
 * one fixed 16 MiB device array inside the library (held on every GPU that loads it until exit);
 * batches that do not fit are rejected with GBO_ERR_OUT_OF_MEMORY (about 44,000 queries for the
 * kinematic-chain metric, more for box spaces). The first call on a device looks the array up
 * (cudaGetSymbolAddress) and must come before any stream capture; every call shares the array, so
 * calls that overlap on the GPU race. Its re-check counters stay in that array: gbo_nn_stats and
 * gbo_nn_error_stats do not include no-alloc calls (folding them in would need a host read). */
gbo_status gbo_nn_nearest_k_noalloc(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, int k,
                                    const int64_t *prefix, int64_t *idx, double *dist, gbo_stream stream);

/* Host-memory drop-ins for NearestNeighbors<T> (AoS rows; synchronous). nearest_r_host answers one
 * query: at most `cap` results are written, *count receives the full count. */
gbo_status gbo_nn_add_host(gbo_nn *nn, const double *states, int64_t n, int64_t *first_key);
gbo_status gbo_nn_remove_host(gbo_nn *nn, const int64_t *keys, int64_t n);
gbo_status gbo_nn_nearest_k_host(gbo_nn *nn, const double *q, int64_t nq, int k, int64_t *idx, double *dist);
gbo_status gbo_nn_nearest_r_host(gbo_nn *nn, const double *q, double r, int64_t cap, int64_t *count, int64_t *idx,
                                 double *dist);
/* Host-memory sampling (AoS rows; synchronous). */
gbo_status gbo_sample_uniform_host(gbo_sampler *s, int64_t n, double *out);
gbo_status gbo_sample_uniform_near_host(gbo_sampler *s, const double *near, double distance, int64_t n, double *out);
gbo_status gbo_sample_gaussian_host(gbo_sampler *s, const double *mean, double stddev, int64_t n, double *out);
gbo_status gbo_sample_valid_host(gbo_sampler *s, gbo_checker *c, int64_t n, unsigned attempts, double *out,
                                 uint8_t *ok);

/* ---- serving ----
 * A request loop for many concurrent planner instances: clients submit validity, motion and nearestK
 * requests over their own device-resident worlds (checkers) and indices (gbo_nn); the server admits a
 * request when a stream slot is free and its device footprint (inputs, outputs) fits in the server's
 * arena, runs admitted requests concurrently on its streams, and frees slots and memory as requests
 * complete (requests behind a blocked one are admitted when they fit). Inputs and outputs are host
 * arrays (AoS rows). gbo_server_submit copies the inputs into the server's page-locked staging
 * arena when it has room (up to 2 GiB, at most the device arena's size), and results reach the
 * caller's arrays when the request completes; without room the request reads and writes the caller's
 * arrays directly, which is slower. Requests on one nearest-neighbour index run one at
 * a time (they share its scratch). No OMPL counterpart: OMPL's planners call the plugins one state at
 * a time from their own threads (tools/multiplan/ParallelPlan.h, geometric/planners/rrt/pRRT.h,
 * geometric/planners/cforest/CForest.h). */
typedef struct gbo_server gbo_server;
enum { GBO_REQ_VALIDITY = 0, GBO_REQ_MOTION = 1, GBO_REQ_KNN = 2 };
typedef struct {
    int kind;                 /* GBO_REQ_* */
    gbo_checker *checker;     /* VALIDITY, MOTION */
    gbo_nn *nn;               /* KNN */
    const double *states;     /* VALIDITY states / MOTION s1 / KNN queries: n rows of dim doubles */
    const double *states2;    /* MOTION s2 */
    int64_t n;
    int k;                    /* KNN */
    int schedule;             /* MOTION: GBO_SCHEDULE_* (AUTO resolves to the checker's tuned choice) */
    uint8_t *ok;              /* VALIDITY / MOTION: n bytes */
    int32_t *first_j;         /* MOTION, nullable */
    int32_t *nd;              /* MOTION, nullable */
    int64_t *idx;             /* KNN: n*k */
    double *dist;             /* KNN: n*k, nullable */
} gbo_request;
gbo_status gbo_server_create(int n_streams, int64_t arena_bytes, gbo_server **out);
gbo_status gbo_server_destroy(gbo_server *s);
/* Queue a request; it runs asynchronously. The arrays must stay valid until gbo_server_wait returns. */
gbo_status gbo_server_submit(gbo_server *s, const gbo_request *req, uint64_t *ticket);
/* Wait for a request (timeout_s < 0: no limit). latency_s: submit-to-completion time. The request's
 * own status is returned (GBO_ERR_TIMEOUT if the wait ran out). */
gbo_status gbo_server_wait(gbo_server *s, uint64_t ticket, double timeout_s, double *latency_s);
gbo_status gbo_server_stats(gbo_server *s, uint64_t *submitted, uint64_t *completed, int64_t *arena_in_use,
                            int *max_concurrent);

/* ---- measurement helper ---- FP32 FMA throughput of this GPU (FLOP/s), for roofline denominators. */
gbo_status gbo_measure_fp32_peak(double *flops, gbo_stream stream);
/* The FP32 cos/sin of the guarded kinematic-chain path for n FP64 angles (device arrays); exposed so
 * that its stated error bound (1.3e-7 per component, |angle| < 100) can be tested against FP64. */
gbo_status gbo_sincos32(const double *theta, int64_t n, float *cos_out, float *sin_out, gbo_stream stream);
/* FP64 FMA throughput of this GPU (FLOP/s). */
gbo_status gbo_measure_fp64_peak(double *flops, gbo_stream stream);
/* Correctly rounded FP64 sin and cos (the device routine of the FP64 forms) of n device values, for
 * tests. No reference counterpart (diagnostic). */
gbo_status gbo_sincos_cr(const double *x, int64_t n, double *sin_out, double *cos_out, gbo_stream stream);
/* FP64 natural log rounded to nearest (the device routine of sampleGaussian's polar method) of n positive
 * normal device values, for tests. No reference counterpart (diagnostic). */
gbo_status gbo_log_rn(const double *x, int64_t n, double *out, gbo_stream stream);
/* Component tags of a PRM roadmap (replaces boost::disjoint_sets in PRM::addMilestone /
 * PRM::uniteComponents, src/ompl/geometric/planners/prm/src/PRM.cpp:580-609, read by
 * PRM::getPlannerData, PRM.cpp:729-756): union_set(src[e], dst[e]) for e = 0..n_edges-1 in order, union
 * by rank with path compression, then root[v] = find_set(v). Host memory only. */
gbo_status gbo_prm_component_roots(const int64_t *src, const int64_t *dst, int64_t n_edges, int64_t n_vertices,
                                   int64_t *root);
/* std::mt19937::discard(J) on a host copy of the generator (no OMPL counterpart; RandomNumbers.h:66-76
 * keeps such a generator): `mt` holds the 624-word block and *pos the index of its next word (1..624,
 * 624 = used up). Afterwards mt / *pos give the same outputs as the original after J draws. Jumps of
 * 1,248 words and more use the jump-ahead polynomial x^J mod phi (phi: the characteristic polynomial of
 * the generator's state transition) instead of stepping; the sampler's large calls use the same jumps
 * on the device. Host memory only. */
gbo_status gbo_mt19937_discard(uint32_t *mt, uint32_t *pos, uint64_t J);
/* Number of kernels this library launched since load (for launch accounting). */
uint64_t gbo_launch_count(void);
/* Self-test of the bounded device waits (no OMPL counterpart): a kernel waits limit_ns nanoseconds
 * (at most 2 s) on a barrier that nothing completes, gives up, and reports it; returns GBO_ERR_TIMEOUT
 * (the expected outcome) with *elapsed_ms the time the wait took. Every device wait of the library
 * (world staging) is bounded the same way (one second) and reports GBO_ERR_TIMEOUT instead of hanging;
 * the context stays usable. */
gbo_status gbo_selftest_bounded_wait(int64_t limit_ns, double *elapsed_ms);

#ifdef __cplusplus
}
#endif
#endif
