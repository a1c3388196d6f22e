/*
 * OMPL plugins backed by libgbompl (include/gbompl.h). Header-only; compile against OMPL's headers
 * and link libgbompl.so. Each class derives from the OMPL interface it replaces:
 *
 *   gbompl::GpuStateValidityChecker   : ompl::base::StateValidityChecker   (StateValidityChecker.h:90-173)
 *   gbompl::GpuDiscreteMotionValidator: ompl::base::MotionValidator        (MotionValidator.h:64-140),
 *                                       DiscreteMotionValidator semantics   (DiscreteMotionValidator.cpp:48-145)
 *   gbompl::GpuStateSampler           : ompl::base::StateSampler           (StateSampler.h:64-108)
 *   gbompl::GpuNearestNeighbors<T>    : ompl::NearestNeighbors<T>          (NearestNeighbors.h:46-115)
 *
 * Single-state virtual calls go through the same batch kernels with n = 1; the batch methods
 * (isValidBatch, checkMotionBatch, sampleUniformBatch, add(vector)) amortise the launch. Errors are
 * raised as ompl::Exception, the exception OMPL itself throws for misconfiguration.
 */
#pragma once

#include <ompl/base/MotionValidator.h>
#include <ompl/base/SpaceInformation.h>
#include <ompl/base/StateSampler.h>
#include <ompl/base/StateValidityChecker.h>
#include <ompl/base/ValidStateSampler.h>
#include <ompl/datastructures/NearestNeighbors.h>
#include <ompl/util/Exception.h>

#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "gbompl.h"

namespace gbompl
{
inline void throwIf(gbo_status s, const char *what)
{
    if (s != GBO_OK)
        throw ompl::Exception(std::string("gbompl: ") + what + ": " + gbo_last_error());
}

/* The GPU objects bound to one OMPL state space: its metric and segment length (read from the OMPL
 * space, never recomputed) and optionally a world for validity checking. */
class GpuContext
{
public:
    /* spaceKind: GBO_SPACE_*; param: link length for GBO_SPACE_KINEMATIC_CHAIN. The OMPL space must be
     * set up (SpaceInformation::setup) so that getLongestValidSegmentLength() is final. */
    GpuContext(ompl::base::StateSpacePtr space, int spaceKind, double param = 0.0) : ompl_(std::move(space))
    {
        dim_ = ompl_->getDimension();
        std::vector<double> lo(dim_, 0.0), hi(dim_, 0.0);
        if (spaceKind == GBO_SPACE_REAL_VECTOR)
        {
            const auto &b = ompl_->as<ompl::base::RealVectorStateSpace>()->getBounds();
            lo = b.low;
            hi = b.high;
        }
        throwIf(gbo_space_create(spaceKind, (int)dim_, lo.data(), hi.data(), param,
                                 ompl_->getLongestValidSegmentLength(), 0.0, ompl_->getValidSegmentCountFactor(),
                                 &space_),
                "space");
    }
    ~GpuContext()
    {
        if (checker_)
            gbo_checker_destroy(checker_);
        gbo_space_destroy(space_);
    }
    GpuContext(const GpuContext &) = delete;
    GpuContext &operator=(const GpuContext &) = delete;

    /* world rows: circles (x, y, r), segments (x0, y0, x1, y1) or spheres (x, y, z, r). */
    void bindWorld(int checkerKind, const std::vector<double> &world, int rowLength, const std::vector<double> &dh = {},
                   int spheresPerLink = 0, double sphereRadius = 0.0, int precision = GBO_PRECISION_FP32_GUARDED)
    {
        if (checker_)
            gbo_checker_destroy(checker_);
        checker_ = nullptr;
        throwIf(gbo_checker_create(space_, checkerKind, world.data(), (int64_t)(world.size() / rowLength),
                                   dh.empty() ? nullptr : dh.data(), (int)(dh.size() / 3), spheresPerLink,
                                   sphereRadius, &checker_),
                "checker");
        throwIf(gbo_checker_set_precision(checker_, precision), "precision");
    }

    gbo_space *space() const { return space_; }
    gbo_checker *checker() const
    {
        if (!checker_)
            throw ompl::Exception("gbompl: no world bound to the GPU context");
        return checker_;
    }
    const ompl::base::StateSpacePtr &omplSpace() const { return ompl_; }
    unsigned dim() const { return dim_; }

    void toRow(const ompl::base::State *s, double *row) const
    {
        auto *st = const_cast<ompl::base::State *>(s);
        for (unsigned i = 0; i < dim_; ++i)
            row[i] = *ompl_->getValueAddressAtIndex(st, i);
    }
    void fromRow(const double *row, ompl::base::State *s) const
    {
        for (unsigned i = 0; i < dim_; ++i)
            *ompl_->getValueAddressAtIndex(s, i) = row[i];
    }

private:
    ompl::base::StateSpacePtr ompl_;
    unsigned dim_ = 0;
    gbo_space *space_ = nullptr;
    gbo_checker *checker_ = nullptr;
};
using GpuContextPtr = std::shared_ptr<GpuContext>;

class GpuStateValidityChecker : public ompl::base::StateValidityChecker
{
public:
    GpuStateValidityChecker(const ompl::base::SpaceInformationPtr &si, GpuContextPtr ctx)
      : ompl::base::StateValidityChecker(si), ctx_(std::move(ctx))
    {
    }
    bool isValid(const ompl::base::State *state) const override
    {
        std::vector<double> row(ctx_->dim());
        ctx_->toRow(state, row.data());
        uint8_t ok = 0;
        throwIf(gbo_is_valid_host(ctx_->checker(), row.data(), 1, &ok), "isValid");
        return ok != 0;
    }
    /* Batch form: out[i] = isValid(states[i]). */
    void isValidBatch(const std::vector<const ompl::base::State *> &states, std::vector<bool> &out) const
    {
        const unsigned d = ctx_->dim();
        std::vector<double> rows(states.size() * d);
        for (size_t i = 0; i < states.size(); ++i)
            ctx_->toRow(states[i], rows.data() + i * d);
        std::vector<uint8_t> ok(states.size());
        throwIf(gbo_is_valid_host(ctx_->checker(), rows.data(), (int64_t)states.size(), ok.data()), "isValid");
        out.assign(ok.begin(), ok.end());
    }

private:
    GpuContextPtr ctx_;
};

class GpuDiscreteMotionValidator : public ompl::base::MotionValidator
{
public:
    GpuDiscreteMotionValidator(const ompl::base::SpaceInformationPtr &si, GpuContextPtr ctx)
      : ompl::base::MotionValidator(si), ctx_(std::move(ctx))
    {
    }
    bool checkMotion(const ompl::base::State *s1, const ompl::base::State *s2) const override
    {
        return one(s1, s2, nullptr);
    }
    bool checkMotion(const ompl::base::State *s1, const ompl::base::State *s2,
                     std::pair<ompl::base::State *, double> &lastValid) const override
    {
        return one(s1, s2, &lastValid);
    }
    /* Batch form over edges (s1[i], s2[i]); lastValidTime[i] as lastValid.second (NaN when valid). */
    void checkMotionBatch(const std::vector<const ompl::base::State *> &s1,
                          const std::vector<const ompl::base::State *> &s2, std::vector<bool> &ok,
                          std::vector<double> *lastValidTime = nullptr) const
    {
        const unsigned d = ctx_->dim();
        const size_t n = s1.size();
        std::vector<double> a(n * d), b(n * d), lt(n);
        for (size_t i = 0; i < n; ++i)
        {
            ctx_->toRow(s1[i], a.data() + i * d);
            ctx_->toRow(s2[i], b.data() + i * d);
        }
        std::vector<uint8_t> r(n);
        throwIf(gbo_check_motion_host(ctx_->checker(), a.data(), b.data(), (int64_t)n, r.data(),
                                      lastValidTime ? lt.data() : nullptr, nullptr),
                "checkMotion");
        ok.assign(r.begin(), r.end());
        std::lock_guard<std::mutex> lk(mu_);
        for (auto v : r)
            (v ? valid_ : invalid_)++;
        if (lastValidTime)
            *lastValidTime = lt;
    }

private:
    bool one(const ompl::base::State *s1, const ompl::base::State *s2,
             std::pair<ompl::base::State *, double> *lastValid) const
    {
        const unsigned d = ctx_->dim();
        std::vector<double> a(d), b(d), ls(d);
        ctx_->toRow(s1, a.data());
        ctx_->toRow(s2, b.data());
        uint8_t ok = 0;
        double lt = 0.0;
        throwIf(gbo_check_motion_host(ctx_->checker(), a.data(), b.data(), 1, &ok, lastValid ? &lt : nullptr,
                                      lastValid && lastValid->first ? ls.data() : nullptr),
                "checkMotion");
        if (!ok && lastValid)
        {
            lastValid->second = lt;
            if (lastValid->first)
                ctx_->fromRow(ls.data(), lastValid->first);
        }
        std::lock_guard<std::mutex> lk(mu_);
        (ok ? valid_ : invalid_)++;
        return ok != 0;
    }
    GpuContextPtr ctx_;
    mutable std::mutex mu_;
};

/* The space's default sampler with its RNG stream on the GPU: the stream of RNG::setLocalSeed(seed)
 * drawn by RealVectorStateSampler / SO2StateSampler, reproduced value for value. */
class GpuStateSampler : public ompl::base::StateSampler
{
public:
    GpuStateSampler(const ompl::base::StateSpace *space, GpuContextPtr ctx, uint32_t localSeed)
      : ompl::base::StateSampler(space), ctx_(std::move(ctx))
    {
        throwIf(gbo_sampler_create(ctx_->space(), localSeed, &s_), "sampler");
    }
    ~GpuStateSampler() override { gbo_sampler_destroy(s_); }
    void sampleUniform(ompl::base::State *state) override
    {
        std::vector<double> row(ctx_->dim());
        throwIf(gbo_sample_uniform_host(s_, 1, row.data()), "sampleUniform");
        ctx_->fromRow(row.data(), state);
    }
    void sampleUniformNear(ompl::base::State *state, const ompl::base::State *near, double distance) override
    {
        std::vector<double> nr(ctx_->dim()), row(ctx_->dim());
        ctx_->toRow(near, nr.data());
        throwIf(gbo_sample_uniform_near_host(s_, nr.data(), distance, 1, row.data()), "sampleUniformNear");
        ctx_->fromRow(row.data(), state);
    }
    void sampleGaussian(ompl::base::State *state, const ompl::base::State *mean, double stdDev) override
    {
        std::vector<double> mr(ctx_->dim()), row(ctx_->dim());
        ctx_->toRow(mean, mr.data());
        throwIf(gbo_sample_gaussian_host(s_, mr.data(), stdDev, 1, row.data()), "sampleGaussian");
        ctx_->fromRow(row.data(), state);
    }
    /* n consecutive sampleUniform draws. */
    void sampleUniformBatch(std::vector<ompl::base::State *> &states)
    {
        const unsigned d = ctx_->dim();
        std::vector<double> rows(states.size() * d);
        throwIf(gbo_sample_uniform_host(s_, (int64_t)states.size(), rows.data()), "sampleUniform");
        for (size_t i = 0; i < states.size(); ++i)
            ctx_->fromRow(rows.data() + i * d, states[i]);
    }

private:
    GpuContextPtr ctx_;
    gbo_sampler *s_ = nullptr;
};

/* UniformValidStateSampler (base/samplers/UniformValidStateSampler.h) on the GPU: sampleUniform draws
 * from the GPU stream of RNG::setLocalSeed(localSeed) until the context's checker reports a valid
 * state or getNrAttempts() draws were made; the stream is consumed exactly as OMPL's sampler would
 * consume it. sampleBatch makes n such calls in one go. */
class GpuUniformValidStateSampler : public ompl::base::ValidStateSampler
{
public:
    GpuUniformValidStateSampler(const ompl::base::SpaceInformation *si, GpuContextPtr ctx, uint32_t localSeed)
      : ompl::base::ValidStateSampler(si), ctx_(std::move(ctx))
    {
        name_ = "uniform";
        throwIf(gbo_sampler_create(ctx_->space(), localSeed, &s_), "sampler");
    }
    ~GpuUniformValidStateSampler() override { gbo_sampler_destroy(s_); }
    bool sample(ompl::base::State *state) override
    {
        std::vector<double> row(ctx_->dim());
        uint8_t ok = 0;
        throwIf(gbo_sample_valid_host(s_, ctx_->checker(), 1, attempts_, row.data(), &ok), "sample");
        ctx_->fromRow(row.data(), state);
        return ok != 0;
    }
    /* UniformValidStateSampler::sampleNear (UniformValidStateSampler.cpp:59-70): sampleUniformNear on
     * the same stream, then isValid, until valid or getNrAttempts() draws were made. */
    bool sampleNear(ompl::base::State *state, const ompl::base::State *near, double distance) override
    {
        const unsigned d = ctx_->dim();
        std::vector<double> c(d), row(d);
        ctx_->toRow(near, c.data());
        uint8_t ok = 0;
        unsigned attempts = 0;
        do
        {
            throwIf(gbo_sample_uniform_near_host(s_, c.data(), distance, 1, row.data()), "sampleNear");
            throwIf(gbo_is_valid_host(ctx_->checker(), row.data(), 1, &ok), "isValid");
            ++attempts;
        } while (!ok && attempts < attempts_);
        ctx_->fromRow(row.data(), state);
        return ok != 0;
    }
    /* states.size() consecutive sample() calls; ok[i] is call i's result. */
    void sampleBatch(std::vector<ompl::base::State *> &states, std::vector<bool> &ok)
    {
        const unsigned d = ctx_->dim();
        std::vector<double> rows(states.size() * d);
        std::vector<uint8_t> r(states.size());
        throwIf(gbo_sample_valid_host(s_, ctx_->checker(), (int64_t)states.size(), attempts_, rows.data(), r.data()),
                "sample");
        for (size_t i = 0; i < states.size(); ++i)
            ctx_->fromRow(rows.data() + i * d, states[i]);
        ok.assign(r.begin(), r.end());
    }

private:
    GpuContextPtr ctx_;
    gbo_sampler *s_ = nullptr;
};

/* The check that a NearestNeighbors distance function (NearestNeighbors.h:58-110) is the state space's
 * own metric, the only one the GPU index evaluates. From setDistanceFunction on, the function is
 * compared with StateSpace::distance on up to 8 consecutive pairs of elements: at once on the stored
 * elements, else on the first elements added afterwards (before they reach the device); a value that
 * differs throws ompl::Exception. Needs no device. */
template <typename T>
class MetricGuard
{
public:
    using DistanceFunction = typename ompl::NearestNeighbors<T>::DistanceFunction;
    MetricGuard(const ompl::base::StateSpace *space, std::function<const ompl::base::State *(const T &)> stateOf)
      : space_(space), stateOf_(std::move(stateOf))
    {
    }
    /* setDistanceFunction(df) with the container's elements `stored`. */
    void set(const DistanceFunction &df, const std::vector<T> &stored)
    {
        df_ = df;
        pending_ = static_cast<bool>(df_);
        check(stored, {});
    }
    /* add(data) with the container's elements `stored`; throws before anything is added. */
    void check(const std::vector<T> &stored, const std::vector<T> &data)
    {
        if (!pending_)
            return;
        std::vector<T> run;
        if (!stored.empty())
            run.push_back(stored.back());
        for (size_t i = 0; i < data.size() && run.size() < 9; ++i)
            run.push_back(data[i]);
        if (data.empty())
            run.assign(stored.begin(), stored.begin() + std::min<size_t>(stored.size(), 9));
        if (run.size() < 2)
            return;
        for (size_t i = 0; i + 1 < run.size(); ++i)
            if (df_(run[i], run[i + 1]) != space_->distance(stateOf_(run[i]), stateOf_(run[i + 1])))
                throw ompl::Exception("gbompl: GpuNearestNeighbors supports the state space's own metric only");
        pending_ = false;
    }

private:
    const ompl::base::StateSpace *space_;
    std::function<const ompl::base::State *(const T &)> stateOf_;
    DistanceFunction df_;
    bool pending_ = false;
};

/* NearestNeighbors<T> over a device-resident index of the elements' states. `stateOf` maps an element
 * to its state (e.g. [](Motion *m) { return m->state; }). Results are ordered by (distance, insertion
 * order). The distance function must be the space's own metric (MetricGuard): a different one throws
 * ompl::Exception from setDistanceFunction or from the first add after it. */
template <typename T>
class GpuNearestNeighbors : public ompl::NearestNeighbors<T>
{
public:
    GpuNearestNeighbors(GpuContextPtr ctx, std::function<const ompl::base::State *(const T &)> stateOf,
                        int64_t capacity = 1 << 20)
      : ctx_(std::move(ctx)), stateOf_(std::move(stateOf)), guard_(ctx_->omplSpace().get(), stateOf_)
    {
        throwIf(gbo_nn_create(ctx_->space(), capacity, &nn_), "nearest neighbours");
    }
    ~GpuNearestNeighbors() override { gbo_nn_destroy(nn_); }

    void setDistanceFunction(const typename ompl::NearestNeighbors<T>::DistanceFunction &df) override
    {
        guard_.set(df, elems_);
        ompl::NearestNeighbors<T>::setDistanceFunction(df);
    }
    bool reportsSortedResults() const override { return true; }
    void clear() override
    {
        throwIf(gbo_nn_clear(nn_), "clear");
        elems_.clear();
        alive_.clear();
    }
    void add(const T &data) override { add(std::vector<T>{data}); }
    void add(const std::vector<T> &data) override
    {
        guard_.check(elems_, data);
        const unsigned d = ctx_->dim();
        std::vector<double> rows(data.size() * d);
        for (size_t i = 0; i < data.size(); ++i)
            ctx_->toRow(stateOf_(data[i]), rows.data() + i * d);
        int64_t first = 0;
        throwIf(gbo_nn_add_host(nn_, rows.data(), (int64_t)data.size(), &first), "add");
        elems_.insert(elems_.end(), data.begin(), data.end());
        alive_.resize(elems_.size(), 1);
    }
    bool remove(const T &data) override
    {
        for (int64_t i = (int64_t)elems_.size() - 1; i >= 0; --i)
            if (alive_[i] && elems_[i] == data)
            {
                throwIf(gbo_nn_remove_host(nn_, &i, 1), "remove");
                alive_[i] = 0;
                return true;
            }
        return false;
    }
    T nearest(const T &data) const override
    {
        std::vector<T> nbh;
        nearestK(data, 1, nbh);
        if (nbh.empty())
            throw ompl::Exception("No elements found in nearest neighbors data structure");
        return nbh[0];
    }
    void nearestK(const T &data, std::size_t k, std::vector<T> &nbh) const override
    {
        nbh.clear();
        if (k == 0)
            return;
        std::vector<double> q(ctx_->dim());
        ctx_->toRow(stateOf_(data), q.data());
        std::vector<int64_t> idx(k);
        throwIf(gbo_nn_nearest_k_host(nn_, q.data(), 1, (int)k, idx.data(), nullptr), "nearestK");
        for (auto i : idx)
            if (i >= 0)
                nbh.push_back(elems_[i]);
    }
    void nearestR(const T &data, double radius, std::vector<T> &nbh) const override
    {
        nbh.clear();
        std::vector<double> q(ctx_->dim());
        ctx_->toRow(stateOf_(data), q.data());
        const int64_t cap = (int64_t)elems_.size();
        std::vector<int64_t> idx(cap + 1);
        std::vector<double> dist(cap + 1);
        int64_t count = 0;
        throwIf(gbo_nn_nearest_r_host(nn_, q.data(), radius, cap, &count, idx.data(), dist.data()), "nearestR");
        for (int64_t i = 0; i < count && i < cap; ++i)
            nbh.push_back(elems_[idx[i]]);
    }
    std::size_t size() const override
    {
        std::size_t c = 0;
        for (auto a : alive_)
            c += a;
        return c;
    }
    void list(std::vector<T> &data) const override
    {
        data.clear();
        for (size_t i = 0; i < elems_.size(); ++i)
            if (alive_[i])
                data.push_back(elems_[i]);
    }

protected:
    GpuContextPtr ctx_;
    std::function<const ompl::base::State *(const T &)> stateOf_;
    MetricGuard<T> guard_;
    gbo_nn *nn_ = nullptr;
    std::vector<T> elems_;
    std::vector<unsigned char> alive_;
};

/* NearestNeighborsSqrtApprox<T> (datastructures/NearestNeighborsSqrtApprox.h) over the same device index:
 * nearest() examines 1 + floor(sqrt(n)) elements chosen round-robin exactly as OMPL's class does (the
 * offset advances per call and restarts at clear()); the other queries are GpuNearestNeighbors'. */
template <typename T>
class GpuNearestNeighborsSqrtApprox : public GpuNearestNeighbors<T>
{
public:
    using GpuNearestNeighbors<T>::GpuNearestNeighbors;
    void clear() override
    {
        GpuNearestNeighbors<T>::clear();
        offset_ = 0;
    }
    T nearest(const T &data) const override
    {
        std::vector<double> q(this->ctx_->dim());
        this->ctx_->toRow(this->stateOf_(data), q.data());
        int64_t key = -1;
        double d = 0.0;
        const gbo_status st = gbo_nn_nearest_sqrt_approx_host(this->nn_, q.data(), 1, &offset_, &key, &d);
        if (st != GBO_OK || key < 0)
            throw ompl::Exception("No elements found in nearest neighbors data structure");
        return this->elems_[key];
    }

private:
    mutable uint64_t offset_ = 0;
};

}  // namespace gbompl
