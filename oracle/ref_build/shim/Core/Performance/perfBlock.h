/* No-op replacement for the reference's Win32-only profiling macros.
 * TEST INFRASTRUCTURE ONLY (CPU oracle build). */
#ifndef PERF_BLOCK_H
#define PERF_BLOCK_H
#include <stdio.h>
#define PERF_BLOCK_MAIN( threadName )
#define PERF_BLOCK_STATIC_MAIN()
#define PERF_BLOCK( label )
#define PERF_BLOCK_ENABLE_PROFILING( numFrames )
#define PERF_BLOCK_CROSS_FRAME_BOUNDARY( tallyEveryFrame )
#define PROFILE_FOREVER -1
#endif
