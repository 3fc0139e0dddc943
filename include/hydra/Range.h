// Range.h -- drop-in header name of the reference for phase_space_range (declared in
// hps_phasespace.hpp); the reference's general Range machinery is not part of this path.
#pragma once
#include "hps_phasespace.hpp"
