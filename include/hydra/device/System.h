// device/System.h -- hydra::device::sys / sys_t (hps_phasespace.hpp).
#pragma once
#include "../hps_phasespace.hpp"
