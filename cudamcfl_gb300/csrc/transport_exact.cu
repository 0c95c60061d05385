/* Exact-math instantiation of the transport kernel (bit-identical to the CPU
 * oracle).  Built with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false. */
#define MCFL_EXACT_MATH 1
#include "transport.cuh"
