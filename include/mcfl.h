/*
 * mcfl.h — C ABI of the GB300 photon-transport engine for voxelized
 * fluorescent turbid media (libmcfl.so).
 *
 * Two layers:
 *
 *  1. The reference's own host interface, as a drop-in.  CUDAMCFL has no
 *     plugin or FFI layer; its boundary is the cuda_fl executable with its
 *     .mci/bulk/output files, and the host routines of CUDAMCFLmain.cu and
 *     CUDAMCFLio.cu.  Each function below names the reference routine it
 *     replaces (file:line in the CUDAMCFL sources).
 *
 *  2. The engine: device-resident media, runs, batches of many sources in
 *     one persistent launch, and a continuous-batching server.
 *
 * Conventions: functions return an int status (MCFL_OK = 0, negative on
 * error) unless stated otherwise; mcfl_last_error() gives the message of the
 * last failure on the calling thread.  The library never prints and never
 * exits.  Buffers are caller-owned.  Images hold nx + nx*ny entries like the
 * reference's (CUDAMCFLmem.cu:113); entry y*nx + x is pixel (x, y).
 */
#ifndef MCFL_H
#define MCFL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  MCFL_OK = 0,
  MCFL_E_ARG = -1,     /* invalid argument */
  MCFL_E_CUDA = -2,    /* CUDA runtime error, or no usable GPU */
  MCFL_E_IO = -3,      /* file could not be opened or written */
  MCFL_E_PARSE = -4,   /* malformed .mci or bulk file */
  MCFL_E_NOMEM = -5,   /* host or device allocation failed */
  MCFL_E_STATE = -6,   /* call not valid in the current state */
  MCFL_E_RANGE = -7,   /* size beyond a supported limit */
  MCFL_E_BUSY = -8,    /* server full: retry later */
  MCFL_E_TIMEOUT = -9, /* wait timed out */
  MCFL_E_CAPPED = -10  /* photons stopped by the per-photon pass cap */
};

#define MCFL_STR_LEN 500
#define MCFL_MAX_BULKS 253
#define MCFL_MAX_LAYERS 98

/* ---------------------------------------------------------------------- */
/* Reference data types                                                    */
/* ---------------------------------------------------------------------- */

/* BulkStruct, CUDAMCFL.h:116-127.  Entry 0 is the medium above the slab,
 * entry n_bulks+1 the medium below; mutr = 1/(mua + mus) or FLT_MAX when
 * mus = 0 (mua of the .mci column, without the fluorophore: the reference's
 * mu_t at both wavelengths).  mua is the excitation absorption
 * (mua + flc*AbsCExi), muaf the emission absorption (mua + flc*AbsCEmi),
 * albedof = mus/(flc*AbsCExi + mus).  mus (not in BulkStruct) is the
 * scattering coefficient: voxel-boundary stepping takes mu_t = mua + mus at
 * excitation and muaf + mus at emission from it (0 with mua = 0: transparent). */
typedef struct mcfl_bulk {
  float mutr, mua, g, n, flc, muaf, eY, albedof;
  float mus;
} mcfl_bulk;

/* LayerStruct, CUDAMCFL.h:38-52 (bulk method 1). */
typedef struct mcfl_layer {
  float z_min, z_max, mutr, mua, g, n, flc, muaf, eY, albedof;
} mcfl_layer;

/* IncStruct, CUDAMCFL.h:98-114 (bulk method 1). */
typedef struct mcfl_inclusion {
  float x, y, z, r, mutr, mua, g, n, flc, muaf, eY, albedof;
} mcfl_inclusion;

/* DetStruct, CUDAMCFL.h:71-96. */
typedef struct mcfl_det {
  float dx, dy, dz;
  int nx, ny, nz;
  float x0, y0, sep;
  float x0_temp_det, y0_temp_det;
  unsigned int x_temp_numdets, y_temp_numdets;
  float x_temp_sepdets, y_temp_sepdets, temp_det_r;
  unsigned int temp_rort;
  unsigned long temp_bins, max_temp;
} mcfl_det;

/* SimulationStruct, CUDAMCFL.h:129-170.  bulk_info holds one uint8 label
 * per voxel (the reference stores short; its parser only produces 0-9). */
typedef struct mcfl_simulation {
  unsigned long long number_of_photons;
  unsigned int number_of_photons_per_voxel;
  unsigned int n_layers;
  unsigned int n_bulks;
  unsigned int start_weight;
  char outp_filename[MCFL_STR_LEN];
  char inp_filename[MCFL_STR_LEN];
  long begin, end;
  char AorB;
  mcfl_det det;
  mcfl_layer *layers;
  mcfl_bulk *bulks;
  mcfl_inclusion inclusion;
  int grid_size;
  float esp;
  float xi, yi, zi, dir;
  float n_down;
  int fhd_activated;
  int do_fl_sim;
  int bulk_method;
  unsigned char *bulk_info;
  char bulkinfo_filename[MCFL_STR_LEN];
  int do_temp_sim;
  /* not in the reference: grid size as the transport computes it, and the
   * number of labels the bulk file held */
  int num_x, num_y, num_z;
  long long bulk_values_read;
} mcfl_simulation;

/* ---------------------------------------------------------------------- */
/* Reference host interface (drop-in)                                      */
/* ---------------------------------------------------------------------- */

/* read_simulation_data, CUDAMCFLio.cu:243-659: parses a .mci file (and the
 * bulk matrix it names, relative to the working directory) into a malloc'ed
 * array.  Returns the number of simulations read, 0 on failure. */
int mcfl_read_simulation_data(const char *filename, mcfl_simulation **simulations, int ignoreAdetection);

/* FreeSimulationStruct, CUDAMCFLmem.cu:219-223. */
void mcfl_free_simulation_struct(mcfl_simulation *simulations, int n_simulations);

/* interpret_arg, CUDAMCFLio.cu:30-55: "-S<seed>" and "-A".  Returns 0, or 1
 * on an unknown argument. */
int mcfl_interpret_arg(int argc, char *argv[], unsigned long long *seed, int *ignoreAdetection);

/* init_RNG, CUDAMCFLrng.cu:31-90: per-stream MWC states and multipliers
 * from a multiplier file.  Returns 0 on success, 1 on failure (as the
 * reference). */
int mcfl_init_RNG(unsigned long long *x, unsigned int *a, unsigned int n_rng, const char *safeprimes_file,
                  unsigned long long xinit);

/* Writes a multiplier file in the format init_RNG reads (the reference does
 * not ship safeprimes_base32.txt): count lines of "a hi lo", a descending
 * from 2^32-1 with a*2^32-1 and a*2^31-1 prime. */
int mcfl_write_safeprimes(const char *path, unsigned int count);

/* DoOneSimulation, CUDAMCFLmain.cu:60-193: excitation run of the .mci's
 * photons with the photon hitting density, on the GPU.  The reference takes
 * per-thread RNG arrays x/a; the engine derives one stream per photon from
 * seed instead.  fhd_out (num_x*num_y*num_z, normalised per photon as
 * CUDAMCFLmain.cu:181-183), Rd_out/Tt_out (raw, det.nx + det.nx*det.ny) may
 * be NULL.  Returns the photons finished, 0 on failure. */
unsigned long long mcfl_DoOneSimulation(const mcfl_simulation *simulation, unsigned long long seed, double *fhd_out,
                                        unsigned long long *Rd_out, unsigned long long *Tt_out);

/* DoOneSimulationFl, CUDAMCFLmain.cu:196-288: one emission run of
 * number_of_photons_per_voxel photons from the voxel whose corner is
 * (xi, yi, zi), isotropic, emission absorption.  Raw R/T images.  Returns
 * the photons finished, 0 on failure. */
unsigned long long mcfl_DoOneSimulationFl(const mcfl_simulation *simulation, unsigned long long seed,
                                          unsigned long long *tempvoxelR, unsigned long long *tempvoxelT);

/* Write_Simulation_Results, CUDAMCFLio.cu:57-191: <out>_param.dat,
 * <out>_Trans.dat, <out>_Refl.dat from raw excitation images. */
int mcfl_Write_Simulation_Results(const mcfl_simulation *sim, const unsigned long long *Rd_xy,
                                  const unsigned long long *Tt_xy, double simulation_time_s);

/* The time-resolved file of Write_Simulation_Results, CUDAMCFLio.cu:168-187
 * (<out>_time.dat): per detector its position and its bins divided by
 * (2^32-1) number_of_photons.  time_xyt: raw tallies as mcfl_run_out. */
int mcfl_write_time(const mcfl_simulation *sim, const unsigned long long *time_xyt);

/* The PHD dump of CUDAMCFLmain.cu:368-392 (<out>_PHD-Ascii.dat). */
int mcfl_write_phd(const mcfl_simulation *sim, const double *fhd);

/* The emission images of CUDAMCFLmain.cu:604-647 (<out>_FlR.dat, _FlT.dat). */
int mcfl_write_fl_images(const mcfl_simulation *sim, const double *flR, const double *flT);

/* main, CUDAMCFLmain.cu:290-668: the whole two-phase run of a .mci file
 * (voxelized or layered medium) with every output file the reference writes,
 * both phases seeded from seed (the reference seeds its emission phase from
 * time(NULL), CUDAMCFLmain.cu:412).  A file with several runs runs all of
 * them, run i seeded from seed + 2i, each writing its own outputs (the
 * reference parses them but simulates only the first).  Paths resolve
 * against the working directory, as the reference's do. */
int mcfl_run_mci(const char *mci_path, unsigned long long seed);

/* ---------------------------------------------------------------------- */
/* Engine                                                                   */
/* ---------------------------------------------------------------------- */

typedef struct mcfl_ctx mcfl_ctx;
typedef struct mcfl_medium mcfl_medium;

/* Kernel numerics. */
enum {
  MCFL_MATH_EXACT = 0, /* IEEE single precision, bit-identical to the CPU oracle */
  MCFL_MATH_FAST = 1,  /* hardware SFU intrinsics (the reference's GPU numerics) */
  MCFL_MATH_F64 = 2    /* the same kernel in double precision: states the single-precision error */
};

/* Source kinds. */
enum {
  MCFL_SOURCE_GAUSS_BEAM = 1, /* the reference's collimated source: radius 0.03 sqrt(-ln u) cm, +z */
  MCFL_SOURCE_WIDEFIELD = 3   /* collimated, uniform over width x height centred on (x, y) */
};

typedef struct mcfl_source {
  int kind;
  float x, y, z;
  float width, height;
} mcfl_source;

/* Voxel grid in the reference's frame: |x| < half_x, |y| < half_y,
 * 0 <= z < thickness; voxel (ix, iy, iz) at index ix + nx*(iy + ny*iz). */
typedef struct mcfl_medium_desc {
  int nx, ny, nz;
  float half_x, half_y, thickness;
  float vox_per_cm[3];          /* inverse voxel sizes */
  const unsigned char *labels;  /* host, nx*ny*nz */
  const float *fluor_map;       /* optional per-voxel emission-strength factor (host, nx*ny*nz), or NULL */
  int n_bulks;                  /* labels 1..n_bulks; 0 above, n_bulks+1 below */
  const mcfl_bulk *bulks;       /* n_bulks + 2 entries */
} mcfl_medium_desc;

typedef struct mcfl_detector {
  float x0, y0, dx, dy;
  int nx, ny;
} mcfl_detector;

/* Time-resolved detectors (the reference's temporal simulation, det.*temp*
 * of CUDAMCFL.h, .mci lines of CUDAMCFLio.cu:374-422, tallies of
 * CUDAMCFLtransport.cu:379-390,406-417): an nx x ny array of discs of radius
 * `radius`, centred on (x0, y0) with separations sep_x, sep_y (detector i at
 * x = i sep_x - (nx - 1) sep_x / 2 + x0), on the entry face (face 0, z = 0) or
 * the exit face (face 1).  A photon leaving through that face inside a disc
 * adds its weight to the disc's bin of its time of flight, `bins` bins over
 * [0, max_fs) femtoseconds; every disc that contains the exit point counts
 * it.  Excitation phase only.  nx = 0: off. */
typedef struct mcfl_time_detectors {
  int nx, ny;
  float x0, y0;
  float sep_x, sep_y;
  float radius;
  int face;
  int bins;
  unsigned long long max_fs;
} mcfl_time_detectors;

/* One two-phase run: excitation from a source, optionally the photon
 * hitting density, optionally the emission phase (photons_per_voxel photons
 * from every voxel whose label has albedof < 1 and whose weight
 * eY (1 - albedof) PHD * fluor_map is non-zero). */
typedef struct mcfl_run_desc {
  unsigned long long photons;
  unsigned int photons_per_voxel; /* 0: no emission phase */
  int fluence;                    /* 1: tally the photon hitting density (forced on for emission) */
  unsigned long long seed_exc, seed_fl;
  unsigned int start_weight;      /* 0: (2^32-1)(1 - R_specular) from n of labels 0 and 1 */
  mcfl_source source;
  mcfl_detector det;
  /* 1: reproduce the reference's first-photon random-number reuse: photons
   * 0..32767 of the excitation run and of each emitting voxel's run draw their
   * first passes from the numbers their launch drew, as each reference thread's
   * first photon does (LaunchPhoton_Global keeps no RNG state,
   * CUDAMCFLtransport.cu:574-581).  This correlates a first photon's launch
   * with its first steps (a small bias, visible mostly in the emission images
   * where 32768 of every voxel's photons are first photons).  0: independent
   * numbers (default of the engine API; the .mci path sets 1). */
  int launch_rng_reuse;
  mcfl_time_detectors tdet; /* mcfl_run only; zero: none */
  /* Index of the excitation run's first photon in the stream family of
   * seed_exc: photon k of the run draws stream photon_offset + k, so runs
   * over disjoint index ranges of one seed (on one GPU or several) sum to the
   * run over their union bit for bit.  0 for a whole run.  With
   * launch_rng_reuse the reuse applies to the photons whose index in the
   * whole run, photon_offset + k, is below 32768, so the shards still sum to
   * the whole run. */
  unsigned long long photon_offset;
  /* 1: voxel-boundary stepping: the optical depth -ln(u) of a pass is spent
   * voxel by voxel with each voxel's mu_t (mua + mus at excitation, muaf +
   * mus at emission: the fluorophore's absorption included), the hitting
   * density and the
   * weight drop use the voxel where the interaction happens, Fresnel acts at
   * every face between different refractive indices with that face's
   * normal, and scattering-free voxels are crossed without interaction.
   * 0: the reference's stepping (the whole pass with the start voxel's mu_t,
   * the label looked up at the end point, z as the Fresnel normal;
   * CUDAMCFLtransport.cu:280-352).  Voxelized media; mcfl_run (excitation
   * and emission, time-resolved detectors included) and mcfl_batch_run over
   * one medium; not through the server or the allocation-free entry. */
  int exact_stepping;
} mcfl_run_desc;

#define MCFL_NSTATS 9
/* stats[]: photons done, passes, absorbed, left at z=0, left at z=esp,
 * roulette loss, roulette gain, zero-drop loss, capped photons (weights in
 * units of 2^-32 of one photon). */

/* Results of a run.  Every pointer may be NULL; sizes in the comments. */
typedef struct mcfl_run_out {
  unsigned long long *Rd, *Tt;       /* raw excitation images (det nx + nx*ny) */
  double *R, *T;                     /* normalised: Rd/((2^32-1) N dx dy) */
  unsigned long long *fhd;           /* raw photon hitting density (voxels) */
  double *phd;                       /* fhd/((2^32-1) N) */
  double *flR, *flT;                 /* emission images, reference normalisation */
  unsigned long long *flR128, *flT128; /* raw emission accumulators, (lo, hi) per pixel */
  unsigned long long stats_exc[MCFL_NSTATS], stats_fl[MCFL_NSTATS];
  unsigned long long photons_fl;     /* emission photons */
  long long fl_voxels;               /* emitting voxels */
  double energy_exc[4];              /* R_all, T_all, absorbed, residual as fractions of the launched weight */
  float ms_exc, ms_fl;               /* GPU time of the two transport launches */
  unsigned long long *time_xyt;      /* raw time-resolved tallies (tdet.nx*tdet.ny*tdet.bins), index
                                        ix + nx*(iy + ny*bin), weights of 2^-32 photon */
} mcfl_run_out;

/* Context on one GPU (device < 0: current device). */
int mcfl_create(int device, mcfl_ctx **ctx);
void mcfl_destroy(mcfl_ctx *ctx);
const char *mcfl_last_error(void);

/* Options: "math" (MCFL_MATH_*), "block" (threads per block, at most the
 * variant's bound), "variant" (occupancy variant of the single-medium kernel:
 * 0 = 256 threads x 4 blocks per SM, 1 = 256 x 5, 2 = 128 x 9; setting it
 * also resets "variant_fl"), "variant_fl" (the emission phase's own
 * occupancy variant in mcfl_run; -1: as "variant"),
 * "mixed_variant" (occupancy variant of the mixed-media kernel that batches
 * over several media and the server run: 0 = 256 x 3, 1 = 256 x 4, the
 * default, 2 = 128 x 7),
 * "blocks_per_sm" (0 = occupancy maximum), "step_cap" (passes per photon),
 * "l2_window" (1: persisting L2 access window on the labels and tallies),
 * "phd_agg" (the photon-hitting-density tally of the single-medium kernel:
 * 0 one atomic add per pass; 1 a thread's successive passes in one voxel
 * summed in a register before the add; 2 the adds of a warp's lanes summed
 * per voxel, one add per distinct voxel; the tallies are the same),
 * "pass_form" (0: the single-medium pass arranged for the SIMT warp, the
 * common case straight-line and every rare case behind one branch; 1: every
 * test of the reference's pass as its own branch; the tallies are the same),
 * "relaunch" (1..32: the lanes of a warp whose photons ended wait until at
 * least this many of them are free, or the warp's tickets are gone, and
 * then start their next photons together; 1 starts each photon as soon as
 * its lane is free; every photon still draws its own stream, so the tallies
 * are the same).
 * The launch shape of the reference is fixed (CUDAMCFL.h:18-20). */
int mcfl_set_option(mcfl_ctx *ctx, const char *key, long long value);
long long mcfl_get_option(mcfl_ctx *ctx, const char *key);

/* Uses a caller stream (cudaStream_t) for all work of this context; NULL
 * restores the context's own stream. */
int mcfl_set_stream(mcfl_ctx *ctx, void *stream);

/* Layered medium with one spherical inclusion: the reference's bulk method 1
 * (LayerStruct/IncStruct of CUDAMCFL.h, transported by MCd,
 * CUDAMCFLtransport.cu:29-239).  layers: n_layers + 2 entries, [1..n_layers]
 * the slabs (z_min, z_max, mutr, mua, g, n as the .mci parser fills them),
 * [0] and [n_layers+1] the media above and below, of which only n is read.
 * The transport is the reference's as it runs: outside the inclusion every
 * step is 1/mu_t itself, not a sampled -ln(u)/mu_t (CUDAMCFLtransport.cu:
 * 87-89); a scattering-free layer or inclusion steps 2 cm; the absorbed
 * weight rounds to nearest and a zero drop does not kill.  The photon hitting
 * density is tallied on the reference's grid (4 esp x 4 esp x esp, grid_size
 * voxels per cm, esp = layers[n_layers].z_max).  Runs on a layered medium are
 * excitation runs (the reference never simulates emission for it), from a
 * collimated source whose z lies in a slab. */
typedef struct mcfl_layered_desc {
  int n_layers;
  const mcfl_layer *layers;
  mcfl_inclusion inclusion;
  int grid_size;
} mcfl_layered_desc;
int mcfl_medium_create_layered(mcfl_ctx *ctx, const mcfl_layered_desc *desc, mcfl_medium **medium);

/* Uploads a medium; it stays resident until mcfl_medium_free, which must
 * come before mcfl_destroy of its context. */
int mcfl_medium_create(mcfl_ctx *ctx, const mcfl_medium_desc *desc, mcfl_medium **medium);
void mcfl_medium_free(mcfl_medium *medium);
size_t mcfl_medium_bytes(const mcfl_medium *medium);

/* Builds the medium of a parsed .mci simulation (bulk method 2). */
int mcfl_medium_from_simulation(mcfl_ctx *ctx, const mcfl_simulation *sim, mcfl_medium **medium);

/* Times every kernel variant with and without the L2 window, with each form
 * of the pass, with "relaunch" 1 and 2 for the SIMT-arranged pass, and (when
 * the run tallies the photon hitting density) with each form of that tally,
 * on a sample of `run` (sample_photons excitation photons,
 * photons_per_voxel scaled by the same fraction) and keeps the fastest in
 * ctx's options ("variant" for the excitation phase, "variant_fl" for the
 * emission phase, "l2_window", "pass_form", "phd_agg", "relaunch"); returns the
 * excitation phase's variant and the photons/s of the kept combination.  No
 * counterpart in the reference. */
int mcfl_autotune(mcfl_ctx *ctx, const mcfl_medium *medium, const struct mcfl_run_desc *run,
                  unsigned long long sample_photons, int *variant, double *photons_per_s);

/* Runs one two-phase simulation and copies the requested results. */
int mcfl_run(mcfl_ctx *ctx, const mcfl_medium *medium, const mcfl_run_desc *run, mcfl_run_out *out);

/* The run description a .mci simulation implies. */
int mcfl_run_desc_from_simulation(const mcfl_simulation *sim, unsigned long long seed, mcfl_run_desc *run);

/* Schedules of many simulations. */
enum {
  MCFL_SCHEDULE_BATCHED = 0, /* all simulations in one persistent launch, replayed as a CUDA graph */
  MCFL_SCHEDULE_PLAIN = 1    /* one launch (and host wait) per simulation, as the reference */
};

/* Runs n excitation-only simulations (sources, budgets, seeds) on one medium,
 * each with its own R/T images; detectors must share nx, ny.  Both schedules
 * give bit-identical images.  outs (n entries, may be NULL) receive the
 * requested images and per-simulation stats; gpu_ms the GPU time of the
 * transport launches. */
int mcfl_batch_run(mcfl_ctx *ctx, const mcfl_medium *medium, const mcfl_run_desc *runs, int n, int schedule,
                   mcfl_run_out *outs, float *gpu_ms);

/* mcfl_batch_run with a medium per simulation (media[i] for runs[i]): many
 * sources, media and budgets in one persistent launch, replayed as a CUDA
 * graph; jobs on different media run the mixed-media kernel variant (each job
 * carries its medium).  Layered media batch only with their own medium. */
int mcfl_batch_run_media(mcfl_ctx *ctx, const mcfl_medium *const *media, const mcfl_run_desc *runs, int n,
                         int schedule, mcfl_run_out *outs, float *gpu_ms);

/* The two-phase run with its emission phase scheduled as the reference's
 * voxel loop does it (CUDAMCFLmain.cu:471-594): one launch and host wait per
 * emitting voxel.  With max_voxels > 0 only the first max_voxels emitting
 * voxels are simulated (to time the schedule on a sample).  Over all voxels
 * the images equal those of mcfl_run bit for bit. */
int mcfl_run_plain(mcfl_ctx *ctx, const mcfl_medium *medium, const mcfl_run_desc *run, long long max_voxels,
                   mcfl_run_out *out);

/* ---------------------------------------------------------------------- */
/* Continuous-batching server                                              */
/* ---------------------------------------------------------------------- */

typedef struct mcfl_server mcfl_server;

typedef struct mcfl_server_opts {
  unsigned long long hbm_budget_bytes; /* admission budget (0: half the free HBM) */
  unsigned int max_jobs;               /* concurrent jobs (0: 64) */
  /* A slice (one launch of the transport kernel over the admitted
   * requests) ends when a request arrives that can be admitted, when a
   * request's last photon finishes, after slice_us microseconds (0: 32000),
   * or after slice_passes transport passes per thread (0: no such cap),
   * whichever comes first. */
  unsigned int slice_passes;
  /* Scheduling of a slice's photon tickets: the oldest admitted request (the
   * head) has a queue of its own; the requests whose remaining photons are
   * at most 1/express_ratio of the head's remaining (0: 8) share an express
   * queue, shortest remaining first, drawn first by one warp in
   * express_period (0: 4); every warp turns to the other queue when its own
   * is empty. */
  unsigned int express_period;
  unsigned int express_ratio;
  unsigned int slice_us;
} mcfl_server_opts;

typedef struct mcfl_server_metrics_t {
  unsigned long long completed;     /* requests finished */
  double p50_ms, p99_ms, max_ms;    /* submit-to-completion latency */
  unsigned long long photons;       /* photons of finished requests */
  unsigned long long slices;        /* persistent-kernel slices launched */
  double busy_s;                    /* wall time spent in slices */
  double span_s;                    /* first submit to last completion */
  double mean_inflight;             /* jobs per slice, mean */
  unsigned long long max_inflight;  /* jobs per slice, maximum */
  unsigned long long hbm_used, hbm_budget;
  double upload_s;                  /* server-thread wall time uploading admitted requests' media */
  double finish_s;                  /* server-thread wall time copying out and releasing finished requests */
  double kernel_s;                  /* GPU time of the slices' transport launches (CUDA events) */
} mcfl_server_metrics_t;

/* Starts the server thread; it owns ctx (and its stream) until
 * mcfl_server_destroy. */
int mcfl_server_create(mcfl_ctx *ctx, const mcfl_server_opts *opts, mcfl_server **server);

/* Queues one request: an excitation run (photons_per_voxel = 0, fluence
 * optional) on its own medium.  Thread-safe.  The medium's host arrays must
 * stay valid until mcfl_server_wait reports the request finished.  Requests
 * larger than the HBM budget finish with MCFL_E_RANGE.  When a slice is
 * running and the request can join the next one, the call ends that slice
 * early with a 4-byte asynchronous copy on a stream of the server's own
 * (made current on the server's device for the call and the caller's
 * device restored). */
int mcfl_server_submit(mcfl_server *server, const mcfl_medium_desc *medium, const mcfl_run_desc *run,
                       unsigned long long *id);

/* Waits for a request (timeout_ms < 0: no limit).  Returns its status, or
 * MCFL_E_TIMEOUT. */
int mcfl_server_wait(mcfl_server *server, unsigned long long id, int timeout_ms);

/* Copies a finished request's raw R/T images, photon hitting density and
 * stats, and forgets the request. */
int mcfl_server_result(mcfl_server *server, unsigned long long id, mcfl_run_out *out, double *latency_ms);

int mcfl_server_metrics(mcfl_server *server, mcfl_server_metrics_t *metrics);

/* Finishes the admitted and queued requests, then stops the thread. */
void mcfl_server_destroy(mcfl_server *server);

/* ---------------------------------------------------------------------- */
/* Allocation-free batch                                                    */
/* ---------------------------------------------------------------------- */

#define MCFL_NOALLOC_MAX_JOBS 64

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (code running inside another framework's memory pool or arena, code
 * that must avoid the synchronisation of cudaMalloc/cudaFree, or code that is
 * only handed device buffers): runs n <= MCFL_NOALLOC_MAX_JOBS excitation
 * simulations on one medium in one persistent launch, like mcfl_batch_run,
 * without allocating anything.  The caller passes the medium on the device
 * (labels, nx*ny*nz bytes, each label <= n_bulks+1: a larger label reads an
 * unset property record; d_prop, 16-byte aligned, 4 floats per label:
 * 1/(mua+mus), mua, g, n for labels 0..n_bulks+1) and the outputs on the
 * device (d_R, d_T: n images of det.nx + det.nx*det.ny 64-bit sums; d_stats:
 * n x MCFL_NSTATS; all three 8-byte aligned), which the call clears.  Every
 * run must give start_weight.  The kernel's scratch (ticket counter, job
 * table, label records, multiplier table, about 159 KB) is one static
 * device array that every GPU loading the library holds until exit; the
 * first call in a CUDA context sets it up, copying the multiplier table
 * synchronously (make it before any stream capture; a new context, e.g.
 * after cudaDeviceReset, is set up again by its first call); calls share the
 * array, so calls that overlap on the GPU race.  The job table is passed to
 * the GPU by value.  Asynchronous on stream (a cudaStream_t, NULL for the
 * default stream).  More than MCFL_NOALLOC_MAX_JOBS runs: MCFL_E_RANGE;
 * misaligned buffers: MCFL_E_ARG. */
int mcfl_batch_run_noalloc(int math, const unsigned char *d_labels, const float *d_prop, int nx, int ny, int nz,
                           float half_x, float half_y, float thickness, const float *vox_per_cm, int n_bulks,
                           const mcfl_run_desc *runs, int n, unsigned long long *d_R, unsigned long long *d_T,
                           unsigned long long *d_stats, void *stream);

/* Kernel launches issued by this context so far. */
unsigned long long mcfl_launch_count(const mcfl_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
