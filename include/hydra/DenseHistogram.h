// DenseHistogram.h -- drop-in header name of the reference for the Dalitz histogram of the examples (Decays::DalitzHistogram)
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
