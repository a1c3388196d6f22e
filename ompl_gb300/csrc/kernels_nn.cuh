// Device-resident nearest-neighbour index arguments and launchers.
#pragma once
#include "kernels.cuh"

namespace gbo
{

struct NNArgs
{
    const double *pts64;        // SoA FP64 elements [dim][cap]
    const float *feat32;        // SoA FP32 features [F][cap]
    const unsigned char *alive; // 1 = present, 0 = removed (tombstone)
    int64_t cap;
    int64_t size;               // keys handed out so far (removed ones included)
    float eps32;                // bound on |distance_fp32 - distance_fp64|
};

void launch_sqrt_approx(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq,
                        int64_t n, int64_t checks, unsigned long long off0, const int64_t *rank, int64_t *idx,
                        double *dist);
void launch_knn_exact(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq, int k,
                      const int64_t *prefix, int64_t *idx, double *dist, const unsigned long long *list,
                      const unsigned long long *list_n, int64_t max_items);
bool launch_knn_fp32(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, const float *qf,
                     int64_t nq, int k, const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                     unsigned long long *fb_n, RunCounters *ctr, float *part_d, int64_t *part_k, int P,
                     const int64_t *qorder, unsigned *thr);
// Cell index of a RealVector / wrapped nearest-neighbour index (large batches, PRM prefix kNN).
struct BoxCellArgs
{
    const int *start;      // [C + 1] first sorted position of each cell
    const int64_t *skey;   // element key at each sorted position
    const float4 *pts8;    // two float4 (8 coordinates) per sorted position
    const float4 *box;     // four float4 per cell: min of coordinates 0-3, 4-7, max 0-3, 4-7
    int C;
};
int bcell_levels(int dim, int64_t n);
void launch_bcell_build(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, int L, int C, int *cell,
                        int *count, int *start, int *fill, int64_t *skey, float4 *pts8, float4 *box);
void launch_bcell_query_order(const LaunchCfg &lc, const SpaceParams &sp, int L, int C, const float *qf, int64_t nq,
                              const int64_t *prefix, int64_t index_n, int bands, int *qcell, int *count, int *start,
                              int *fill, int64_t *qorder);
bool launch_knn_bcell(const LaunchCfg &lc, const NNArgs &nn, const BoxCellArgs &ci, const SpaceParams &sp,
                      StatesView qv, const float *qf, int64_t nq, const int64_t *qorder, const int *qcell, int k,
                      const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                      unsigned long long *fb_n, RunCounters *ctr, float *part_d, int64_t *part_k);

// Spatial processing order of a query batch (counting sort by a cell key of its FP32 features):
// work holds 3 * kQueryKeys + nq ints, order nq entries.
constexpr int kQueryKeys = 4096;
void launch_query_order(const LaunchCfg &lc, const SpaceParams &sp, const float *qf, int64_t nq, int *work,
                        int64_t *order);
// Cell index of a kinematic-chain nearest-neighbour index (large batches without prefix limits):
// kQueryKeys cells keyed like the query order.
struct ChainCellArgs
{
    const int *start;      // [kQueryKeys] first sorted position of each cell
    const int *count;      // [kQueryKeys] elements per cell
    const int64_t *skey;   // element key at each sorted position
    const float4 *sfeat;   // five planes of float4 (features 4j..4j+3 of each sorted position in plane j)
    int64_t fs;            // plane stride (float4 units)
    const uint4 *box;      // five uint4 per cell: feature f's (minimum, maximum) as a half2 rounded outward
    const int *cstart;     // [kQueryKeys + 1] first chunk of each cell (chunks of 32 sorted positions)
    const uint4 *cbox;     // five uint4 per chunk, as box
};
// key: [size] ints; count / start / fill: [kQueryKeys] ints; skey: [size]; sfeat: 5 planes of [size]; box: [5 * kQueryKeys];
// cstart: [kQueryKeys + 1]; cbox: [5 * (size / 32 + kQueryKeys)]
void launch_ccell_build(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, int *key, int *count,
                        int *start, int *fill, int64_t *skey, float4 *sfeat, uint4 *box, int *cstart, uint4 *cbox);
// qorder / qkey: the query order and each query's key (launch_query_order's order and key arrays).
// Returns true when launched (lists for every query, P = 1, and the finish kernel).
bool launch_knn_ccell(const LaunchCfg &lc, const NNArgs &nn, const ChainCellArgs &ci, const SpaceParams &sp,
                      StatesView qv, const float *qf, int64_t nq, const int64_t *qorder, const int *qkey, int k,
                      int64_t *idx, double *dist, unsigned long long *fb_list, unsigned long long *fb_n,
                      RunCounters *ctr, float *part_d, int64_t *part_k);

int knn_chunks(const LaunchCfg &lc, int64_t nq, int64_t size);
// largest k of the FP32-guarded kNN forms (64 for box / wrapped kinds of dim <= 8, else 20; larger k
// and other kinds use the FP64 scan) and the list length they keep per query and chunk
int knn_fp32_max_k(const SpaceParams &sp);
int knn_keep(int k);
void launch_features(const LaunchCfg &lc, const SpaceParams &sp, StatesView v, int64_t n, float *out, int64_t ld_out);
void launch_store_points(const LaunchCfg &lc, StatesView v, int64_t n, int dim, double *pts, int64_t cap,
                         int64_t first, unsigned char *alive);
void launch_remove(const LaunchCfg &lc, const int64_t *keys, int64_t n, int64_t size, unsigned char *alive);
void launch_radius(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq, double r,
                   int64_t *counts, const int64_t *offsets, int64_t *idx, double *dist);

// sampler
struct SamplerState
{
    unsigned int mt[624];
    unsigned int pos;        // next word index in mt (624 = twist needed)
    unsigned int has_saved;  // normal_distribution's cached second value of the last polar pair
    double saved;
};
// Progress of one chunk of a Gaussian sampling call (device memory, read back by the host)
struct GaussChunk
{
    long long accepted;  // accepted candidates of the chunk
    long long consumed;  // stream words used: through the last needed accepted candidate, else all
    long long slow;      // pairs log_fast leaves (gauss_slow_kernel)
    long long slow_cr;   // pairs log_med leaves too (gauss_cr_kernel)
};
// words: scratch of cap_words (even, >= 2) 32-bit words; calls above cap_words / 2 values run in chunks
void launch_sample_uniform(const LaunchCfg &lc, SamplerState *st, const SpaceParams &sp, const double *near,
                           StatesView nearv, double distance, int64_t n, MutStatesView out, unsigned *words,
                           int64_t cap_words);
// Segmented form of the call (jump-ahead; kernels_sample.cu): nseg segments of L words, windows 1..nseg-1
// from the jump polynomials `polys` (x^(sL) mod phi, mt_jump.cu); scratch of sample_jump_words(nseg, W).
void launch_sample_uniform_jump(const LaunchCfg &lc, SamplerState *st, const SpaceParams &sp, const double *near,
                                StatesView nearv, double distance, int64_t n, MutStatesView out, unsigned *scratch,
                                const uint32_t *polys, int64_t L, int nseg);
int64_t sample_jump_words(int64_t nseg, int64_t W);
bool mt_field_ready();
gbo_status mt_jump_table(uint64_t L, int K, const uint32_t **out);
// sampleGaussian values [v_first, M) of a call; st->has_saved says whether value 0 is the cached one.
// One chunk of at most cap_words / 4 - 156 polar candidates per host round trip; returns the chunks run
// or -1 on an error. words: scratch of cap_words words; ctl: device GaussChunk; cnt: scratch of
// (cap_words / 4096 + 2) long longs; pair / kidx: scratch of gauss_pair_slots(cap_words) entries; slowlist:
// twice that (the pairs log_fast leaves, then those log_med leaves).
int64_t launch_sample_gaussian(const LaunchCfg &lc, SamplerState *st, bool has_saved, const SpaceParams &sp,
                               StatesView meanv, double stddev, int64_t n, MutStatesView out, unsigned *words,
                               int64_t cap_words, GaussChunk *ctl, long long *cnt, double2 *pair,
                               unsigned short *kidx, unsigned *slowlist, unsigned *jump_scratch,
                               const uint32_t *polys, int64_t L);
inline int64_t gauss_pair_slots(int64_t cap_words)
{
    return 1024 * (cap_words / 4096 + 1);
}
// log_rn (the sampleGaussian log, rounded to nearest) of n device values, for tests.
void launch_log_rn(const LaunchCfg &lc, const double *x, int64_t n, double *out);
double measure_fp32_peak(const LaunchCfg &lc);
double measure_fp64_peak(const LaunchCfg &lc);
void launch_sincos32(const LaunchCfg &lc, const double *theta, int64_t n, float *c, float *s);

}  // namespace gbo
