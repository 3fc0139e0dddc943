// host/System.h -- hydra::host::sys / sys_t (hps_phasespace.hpp).
#pragma once
#include "../hps_phasespace.hpp"
