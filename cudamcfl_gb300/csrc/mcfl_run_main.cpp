/*
 * mcfl_run — drop-in for the reference's cuda_fl program (CUDAMCFLmain.cu:290-668):
 *
 *   mcfl_run <file.mci> [-S<seed>] [-A]
 *
 * Reads the .mci file and its bulk matrix (paths relative to the working
 * directory), runs excitation with the photon hitting density and, when the
 * file asks for it, the emission phase on the GPU, and writes
 * <out>_param.dat, _Refl.dat, _Trans.dat, _PHD-Ascii.dat, _FlR.dat and
 * _FlT.dat.  Unlike the reference, both phases are seeded from -S (or the
 * clock), and the exit status reports failure.
 */
#include <cstdio>
#include <ctime>

#include "mcfl.h"

int main(int argc, char *argv[]) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <file.mci> [-S<seed>] [-A]\n", argv[0]);
    return 1;
  }
  unsigned long long seed = (unsigned long long)std::time(nullptr);
  int ignoreA = 0;
  if (mcfl_interpret_arg(argc, argv, &seed, &ignoreA)) {
    std::fprintf(stderr, "%s\n", mcfl_last_error());
    return 1;
  }
  const int rc = mcfl_run_mci(argv[1], seed);
  if (rc != MCFL_OK) {
    std::fprintf(stderr, "mcfl_run: %s (status %d)\n", mcfl_last_error(), rc);
    return 1;
  }
  return 0;
}
