// Function.h -- drop-in header name of the reference for hydra::Function's functor base; functors here are any callable taking the event tuple
// (declared in hps_phasespace.hpp).
#pragma once
#include "hps_phasespace.hpp"
