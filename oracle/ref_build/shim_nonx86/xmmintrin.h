/* Stand-in for the x86 SSE header on hosts without it.  The reference includes
 * it in FluidBodySim/fluidBodySim.cpp but uses no SSE intrinsic there (the one
 * _mm_prefetch is commented out).  CPU oracle build only. */
#pragma once
