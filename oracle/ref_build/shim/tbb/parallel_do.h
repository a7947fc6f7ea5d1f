/* Forwarding header for the std::thread TBB stand-in (CPU oracle build only). */
#pragma once
#include "vg_tbb.h"
