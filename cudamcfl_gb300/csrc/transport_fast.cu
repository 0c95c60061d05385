/* Fast-math instantiation of the transport kernel: hardware SFU intrinsics,
 * the numerics of the reference's own GPU build.  Built with --use_fast_math. */
#define MCFL_EXACT_MATH 0
#include "transport.cuh"
