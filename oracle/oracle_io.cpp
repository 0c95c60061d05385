/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (see oracle/README.md).
 *
 * Writers that CUDAMCFLmain.cu performs inline (and that ref_driver.cpp
 * therefore restates): the photon-hitting-density dump
 * (CUDAMCFLmain.cu:368-392) and the emission images (CUDAMCFLmain.cu:604-647).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_api.h"

extern "C" int oracle_write_phd(const char *prefix, const double *fx, int nx, int ny, int nz) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_PHD-Ascii.dat", prefix);
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  /* CUDAMCFLmain.cu:385 prints three ints with %llu; the values are the same */
  fprintf(f, "%llu\t%llu\t%llu\n", (unsigned long long)nx, (unsigned long long)ny, (unsigned long long)nz);
  const long n = (long)nx * ny * nz;
  for (long i = 0; i < n; ++i) fprintf(f, "%.10E\n", fx[i]);
  fclose(f);
  return 0;
}

static int write_image(const char *path, const double *img, int nx, int ny) {
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (int y = 0; y < ny; y++) {
    for (int x = 0; x < nx; x++) fprintf(f, " %E ", img[y * nx + x]);
    fprintf(f, " \n ");
  }
  fclose(f);
  return 0;
}

extern "C" int oracle_write_fl_images(const char *prefix, const double *flR, const double *flT, int nx, int ny) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_FlR.dat", prefix);
  if (write_image(path, flR, nx, ny)) return -1;
  snprintf(path, sizeof(path), "%s_FlT.dat", prefix);
  return write_image(path, flT, nx, ny);
}

extern "C" void oracle_free_result(oracle_result *r) {
  free(r->Rd); free(r->Tt); free(r->fhd); free(r->flR); free(r->flT);
  free(r->flR128); free(r->flT128); free(r->time_xyt);
  memset(r, 0, sizeof(*r));
}
