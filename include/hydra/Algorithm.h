// Algorithm.h -- drop-in header name of the reference for the reference's algorithm header; the phase-space algorithms are members of PhaseSpace and Decays
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
