/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (see oracle/README.md).
 *
 * C interface shared by the two CPU oracles:
 *   ref_*     the reference's own transport compiled for the host
 *             (ref_driver.cpp; built only where the reference checkout exists)
 *   oracle_*  the restatement of the same algorithm (port.cpp), which also
 *             runs the photon-indexed variant that the CUDA engine implements.
 */
#ifndef MCFL_ORACLE_API_H
#define MCFL_ORACLE_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Result of one two-phase run (excitation + photon hitting density, then the
 * emission images).  Arrays are malloc'ed; free with oracle_free_result. */
typedef struct oracle_result {
  int grid[3];  /* voxels in x, y, z */
  int image[2]; /* detector pixels nx, ny; image arrays hold nx + nx*ny entries */
  unsigned long long number_of_photons;
  unsigned long long photons_exc; /* excitation photons finished */
  unsigned long long photons_fl;  /* emission photons finished (all emitting voxels) */
  long fl_voxels;                 /* emitting voxels simulated */
  long failed_voxels;             /* emission simulations that hit the relaunch cap */
  unsigned long long *Rd, *Tt;    /* raw excitation R/T images, 32-bit weights summed in 64 bits */
  unsigned long long *fhd;        /* raw photon hitting density per voxel */
  double *flR, *flT;              /* emission images in the reference's normalisation */
  /* photon-indexed variant only: raw 128-bit emission accumulators (lo, hi) */
  unsigned long long *flR128, *flT128;
  /* photon-indexed variant only: exact weight accounting of the excitation
   * phase: absorbed, left through z=0, left through z=esp, lost to roulette,
   * gained by roulette, killed by a zero weight drop */
  unsigned long long balance[6];
  unsigned long long steps_exc, steps_fl;
  /* time-resolved detectors of the excitation phase (when enabled): raw
   * weights per detector and time bin, index ix + nx*(iy + ny*bin) */
  unsigned long long *time_xyt;
  long time_size;
  /* reference streams: wall-clock seconds of the excitation phase and of the
   * emission phase (every emitting voxel) */
  double seconds_exc, seconds_fl;
} oracle_result;

/* Parsed method-2 simulation (the fields of SimulationStruct that the
 * transport and the fluorescence driver read, CUDAMCFL.h:116-170). */
#define ORACLE_MAX_BULKS 100
typedef struct oracle_bulk {
  float mutr, mua, g, n, flc, muaf, eY, albedof;
  float mus; /* scattering coefficient: mu_t of voxel-boundary stepping */
} oracle_bulk;

#define ORACLE_MAX_LAYERS 100
typedef struct oracle_layer {
  float z_min, z_max, mutr, mua, g, n, flc, muaf, eY, albedof;
} oracle_layer;
typedef struct oracle_inclusion {
  float x, y, z, r, mutr, mua, g, n, flc, muaf, eY, albedof;
} oracle_inclusion;

typedef struct oracle_sim {
  unsigned long long number_of_photons;
  unsigned int number_of_photons_per_voxel;
  unsigned int n_bulks;
  unsigned int start_weight;
  int grid_size;
  float esp;
  float xi, yi, zi, dir;
  int fhd_activated;
  int do_fl_sim;
  int bulk_method;
  /* detector */
  float det_dx, det_dy;
  int det_nx, det_ny;
  float det_x0, det_y0;
  oracle_bulk bulks[ORACLE_MAX_BULKS + 2];
  const short *bulk_info; /* num_x*num_y*num_z labels, x fastest */
  /* Optional general geometry (not expressible in a .mci file): when nx > 0
   * the grid is nx*ny*nz voxels, |x| < half_x, |y| < half_y, 0 <= z < esp,
   * with vox_per_cm voxels per cm per axis.  Otherwise the reference's
   * geometry: half extents 2*esp and grid_size voxels per cm. */
  int nx, ny, nz;
  float half_x, half_y;
  float vox_per_cm[3];
  const float *fluor_map; /* optional emission-strength factor per voxel (both RNG schemes) */
  long max_fl_voxels;     /* refstream only: stop after this many emitting voxels (0: all) */
  int launch_rng_reuse;   /* photon only: photons 0..32767 of a run (of each voxel) restart their stream
                             after launch, as each reference thread's first photon does */
  /* Time-resolved detectors (CUDAMCFL.h det.*temp*; .mci lines of
   * CUDAMCFLio.cu:374-422): a tdet_nx x tdet_ny array of discs of radius
   * tdet_r centred on (tdet_x0, tdet_y0) with separations tdet_sep_*, on the
   * entry (tdet_face 0) or exit face (1); tdet_bins bins over [0, tdet_max)
   * femtoseconds of time of flight.  Excitation phase only. */
  int do_temp_sim;
  float tdet_x0, tdet_y0;
  int tdet_nx, tdet_ny;
  float tdet_sep_x, tdet_sep_y;
  float tdet_r;
  int tdet_face;
  long tdet_bins;
  unsigned long long tdet_max;
  /* Bulk method 1 (CUDAMCFL.h LayerStruct/IncStruct; .mci lines of
   * CUDAMCFLio.cu:424-511): n_layers slabs (layers[1..n_layers], with
   * layers[0] and layers[n_layers+1] the media above and below, of which only
   * n is read) and one spherical inclusion. */
  int n_layers;
  oracle_layer layers[ORACLE_MAX_LAYERS + 2];
  oracle_inclusion inclusion;
  /* photon only: index of the excitation run's first photon in its stream
   * family (runs over disjoint index ranges sum to the run over their union) */
  unsigned long long photon_offset;
  /* photon only, voxelized media: 1 = voxel-boundary ("exact") stepping
   * instead of the reference's whole-step-in-the-start-voxel transport */
  int exact_stepping;
} oracle_sim;

/* The free-radius map of voxel-boundary stepping (port.cpp free_radius). */
void oracle_free_radius(const short *labels, unsigned nx, unsigned ny, unsigned nz, unsigned char *out);
void oracle_free_result(oracle_result *r);

/* Reference build (oracle/_ref).  seed_fl replaces time(NULL) of the emission
 * phase.  nthreads > 1 trades reproducibility for speed. */
int ref_run_mci(const char *mci_path, const char *safeprimes_path, unsigned long long seed_exc,
                unsigned long long seed_fl, int nthreads, int write_files, oracle_result *res);
/* The reference's own .mci parser, flattened into oracle_sim.  bulk_info is
 * malloc'ed and owned by the caller. */
int ref_parse_mci(const char *mci_path, oracle_sim *out);

/* Restatement, reference RNG streams (32768 per-thread MWC streams seeded by
 * init_RNG from the multiplier file, one sequential schedule).  With
 * math_libm=1 it reproduces ref_run_mci bit for bit. */
int oracle_run_refstream(const oracle_sim *sim, const char *safeprimes_path, unsigned long long seed_exc,
                         unsigned long long seed_fl, int math_libm, int nthreads, oracle_result *res);

/* Restatement, photon-indexed streams (the CUDA engine's scheme): photon k of
 * a phase draws from an MWC stream derived from (seed, phase, k); emission is
 * one job over all emitting voxels with fixed-point voxel weights.  With
 * math_libm=0 it is bit-identical to the CUDA engine's exact-math kernel. */
int oracle_run_photon(const oracle_sim *sim, const uint32_t *multipliers, unsigned int n_multipliers,
                      unsigned long long seed_exc, unsigned long long seed_fl, int math_libm, int nthreads,
                      oracle_result *res);

/* Writers of the emission images in the reference's text format
 * (CUDAMCFLmain.cu:604-647). */
int oracle_write_phd(const char *prefix, const double *fx, int nx, int ny, int nz);
int oracle_write_fl_images(const char *prefix, const double *flR, const double *flT, int nx, int ny);

int oracle_safeprime_multipliers(uint32_t *out, int count);
int oracle_write_safeprimes(const char *path, int count);

#ifdef __cplusplus
}
#endif
#endif
