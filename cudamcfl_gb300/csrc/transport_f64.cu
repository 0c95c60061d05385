/* Double-precision instantiation of the transport kernel: every position,
 * direction, step length and probability in FP64 with IEEE double functions,
 * on the same photon streams and integer tallies.  It exists to state the
 * error of the single-precision kernels; built without fast-math flags. */
#define MCFL_EXACT_MATH 1
#define MCFL_F64 1
#include "transport.cuh"
