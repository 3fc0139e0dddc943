// PhaseSpaceIntegrator.h -- drop-in header name of the reference; the classes live in hps_phasespace.hpp.
#pragma once
#include "hps_phasespace.hpp"
