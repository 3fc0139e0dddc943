// Placeholders.h -- drop-in header name of the reference for hydra::placeholders::_0 ... _9
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
