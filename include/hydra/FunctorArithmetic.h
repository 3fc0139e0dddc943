// FunctorArithmetic.h -- drop-in header name of the reference for functor arithmetic; the phase-space path takes each functor on its own
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
