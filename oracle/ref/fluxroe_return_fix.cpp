// Definitions of the explicit specialisations declared in fluxroe_return_fix.hpp.
// TEST INFRASTRUCTURE ONLY.  Each one stores the Roe-averaged velocity component iDim,
// accumulates its square into Q_SQ and its normal projection into V_CONTRAVARIANT exactly
// as src/FluxRoe.tpp:93-105 of joel-ho/BES does, and then returns the stored component.
#include "fluxroe_return_fix.hpp"

#define BES_REF_ROE_VELOCITY(TYPE)                                                          \
  template <>                                                                               \
  TYPE FluxRoe_<TYPE>::computeRoeAveragedVelocity_(const short iDim, const TYPE denominator, \
                                                   double const* nonDimNormal) {            \
    const short k = mapRoeVelocityComponent_(iDim);                                         \
    roeAveragedVariable_[k] =                                                               \
        (computeNumerator_(this->config_->getPrimitiveVariableVelocityComponent(iDim)) /    \
         denominator);                                                                      \
    roeAveragedVariable_[mapRoeVariable_(FlowVariable::Q_SQ)] +=                            \
        (roeAveragedVariable_[k] * roeAveragedVariable_[k]);                                \
    roeAveragedVariable_[mapRoeVariable_(FlowVariable::V_CONTRAVARIANT)] +=                 \
        (roeAveragedVariable_[k] * nonDimNormal[iDim]);                                     \
    return roeAveragedVariable_[k];                                                         \
  }

BES_REF_ROE_VELOCITY(double)
BES_REF_ROE_VELOCITY(BesRefAd3d)
BES_REF_ROE_VELOCITY(BesRefAd2d)
