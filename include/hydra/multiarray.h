// multiarray.h -- drop-in header name of the reference for hydra::multiarray; Evaluate's result columns are hydra::multivector
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
