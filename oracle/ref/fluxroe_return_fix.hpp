// Force-included (g++ -include) into every translation unit of the patched reference
// build.  TEST INFRASTRUCTURE ONLY.
//
// FluxRoe_<T>::computeRoeAveragedVelocity_ (src/FluxRoe.tpp:90-107 of joel-ho/BES) is
// declared to return T but has no return statement; g++ >= 8 treats the fall-through as
// unreachable and the build crashes on the first Roe flux.  Its return value is never
// used (call site src/FluxRoe.tpp:128).  Instead of editing the reference sources, this
// header declares explicit specialisations of that one member for every T the reference
// instantiates (double, and the Eigen AutoDiff scalars of the 2-D and 3-D Roe Jacobians),
// so the generic body is never instantiated; fluxroe_return_fix.cpp defines them with the
// same arithmetic plus the missing return.
#pragma once
#include "FluxJacobianWrapper.hpp"

typedef Eigen::AutoDiffScalar<Eigen::Matrix<double, 10, 1> > BesRefAd3d;
typedef Eigen::AutoDiffScalar<Eigen::Matrix<double, 8, 1> > BesRefAd2d;

template <>
double FluxRoe_<double>::computeRoeAveragedVelocity_(const short iDim, const double denominator,
                                                     double const* nonDimNormal);
template <>
BesRefAd3d FluxRoe_<BesRefAd3d>::computeRoeAveragedVelocity_(const short iDim,
                                                             const BesRefAd3d denominator,
                                                             double const* nonDimNormal);
template <>
BesRefAd2d FluxRoe_<BesRefAd2d>::computeRoeAveragedVelocity_(const short iDim,
                                                             const BesRefAd2d denominator,
                                                             double const* nonDimNormal);
