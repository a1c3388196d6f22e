/*
 * ORACLE (test infrastructure only): empty definitions for out-of-line members that OMPL's
 * state-space sources reference but that sit off the sampling / validity / motion / kNN path
 * (default projections, used by planners such as KPIECE; the prolate hyperspheroid, used by
 * informed sampling). Their real definitions need Eigen's decompositions, which the oracle build
 * does not have. None of them is ever called by the oracle.
 */
#include "ompl/base/ProjectionEvaluator.h"
#include "ompl/base/spaces/RealVectorStateProjections.h"
#include "ompl/util/ProlateHyperspheroid.h"

namespace ompl
{
unsigned int ProlateHyperspheroid::getDimension() const { return 0; }
void ProlateHyperspheroid::transform(const double *, double *) const {}
namespace base
{
ProjectionMatrix::Matrix ProjectionMatrix::ComputeRandom(unsigned int, unsigned int, const std::vector<double> &) { return {}; }
ProjectionMatrix::Matrix ProjectionMatrix::ComputeRandom(unsigned int, unsigned int) { return {}; }
void ProjectionMatrix::computeRandom(unsigned int, unsigned int, const std::vector<double> &) {}
void ProjectionMatrix::computeRandom(unsigned int, unsigned int) {}
void ProjectionMatrix::project(const double *, Eigen::Ref<Eigen::VectorXd>) const {}
void ProjectionMatrix::print(std::ostream &) const {}
ProjectionEvaluator::ProjectionEvaluator(const StateSpace *space)
  : space_(space), bounds_(0), estimatedBounds_(0), defaultCellSizes_(true), cellSizesWereInferred_(false) {}
ProjectionEvaluator::ProjectionEvaluator(const StateSpacePtr &space) : ProjectionEvaluator(space.get()) {}
ProjectionEvaluator::~ProjectionEvaluator() = default;
bool ProjectionEvaluator::userConfigured() const { return false; }
void ProjectionEvaluator::defaultCellSizes() {}
void ProjectionEvaluator::setCellSizes(const std::vector<double> &) {}
void ProjectionEvaluator::setup() {}
void ProjectionEvaluator::printSettings(std::ostream &) const {}
void ProjectionEvaluator::printProjection(const Eigen::Ref<Eigen::VectorXd> &, std::ostream &) const {}
RealVectorLinearProjectionEvaluator::RealVectorLinearProjectionEvaluator(const StateSpace *space, const std::vector<double> &, const ProjectionMatrix::Matrix &) : ProjectionEvaluator(space) {}
RealVectorLinearProjectionEvaluator::RealVectorLinearProjectionEvaluator(const StateSpace *space, const ProjectionMatrix::Matrix &) : ProjectionEvaluator(space) {}
unsigned int RealVectorLinearProjectionEvaluator::getDimension() const { return 0; }
void RealVectorLinearProjectionEvaluator::project(const State *, Eigen::Ref<Eigen::VectorXd>) const {}
RealVectorIdentityProjectionEvaluator::RealVectorIdentityProjectionEvaluator(const StateSpace *space) : ProjectionEvaluator(space) {}
unsigned int RealVectorIdentityProjectionEvaluator::getDimension() const { return 0; }
void RealVectorIdentityProjectionEvaluator::defaultCellSizes() {}
void RealVectorIdentityProjectionEvaluator::setup() {}
void RealVectorIdentityProjectionEvaluator::project(const State *, Eigen::Ref<Eigen::VectorXd>) const {}
}
}
