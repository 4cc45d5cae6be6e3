// Stand-in for the libconfig++ header so that the reference sources compile
// into the oracle build (oracle/_ref).  It maps the libconfig++ API onto the
// package's own libconfig-format reader (csrc/host/libconfig_lite.hpp); no
// arithmetic of the simulation passes through it.
#pragma once
#include "libconfig_lite.hpp"
