// Lambda.h -- drop-in header name of the reference for hydra::wrap_lambda / hydra::Lambda
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
