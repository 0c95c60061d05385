/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (see oracle/README.md).
 *
 * Host driver that runs the reference's own transport code on the CPU.  The
 * reference sources are compiled in place from the reference checkout (the
 * include path is given by oracle/Makefile); nothing of them is copied here.
 * ref_shim.h supplies the CUDA intrinsics.
 *
 * CUDAMCFLmain.cu cannot be compiled by a host compiler (<<<>>> launches), so
 * this file restates its three host routines:
 *   DoOneSimulation    CUDAMCFLmain.cu:60-193   excitation + photon hitting density
 *   DoOneSimulationFl  CUDAMCFLmain.cu:196-288  one emission simulation
 *   the voxel loop     CUDAMCFLmain.cu:409-652  two-phase fluorescence image
 * A kernel launch <<<128,256>>> becomes a loop over the 32768 virtual threads.
 * With one host thread the loop runs block by block, thread by thread, which is
 * one valid schedule of the GPU kernel and makes every result reproducible;
 * with several host threads the blocks are dealt out round-robin and the
 * results are those of another valid schedule (used for timing only).
 *
 * Deviations from CUDAMCFLmain.cu, all for reproducibility or memory safety:
 *   - the emission phase is seeded from the caller instead of time(NULL)
 *     (CUDAMCFLmain.cu:412);
 *   - the per-voxel image buffers are zeroed (CUDAMCFLmain.cu:501-506 leaves
 *     them uninitialised and multiplies them by 0 when a voxel is skipped);
 *   - nothing is printed.
 */
#include "CUDAMCFL.h"

#include <atomic>
#include <thread>
#include <vector>

thread_local mcfl_shim_dim3 blockIdx;
thread_local mcfl_shim_dim3 threadIdx;

/* The constant-memory symbols of CUDAMCFLmain.cu:34-52, as host globals. */
unsigned long long num_photons_dc[1];
unsigned int n_layers_dc[1];
unsigned int n_bulks_dc[1];
unsigned int start_weight_dc[1];
LayerStruct layers_dc[MAX_LAYERS];
BulkStruct bulks_dc[MAX_LAYERS];
DetStruct det_dc[1];
IncStruct inclusion_dc[1];
unsigned int ignoreAdetection_dc[1];
unsigned int fhd_activated_dc[1];
unsigned int do_temp_sim_dc[1];
unsigned int bulk_method_dc[1];
float xi_dc[1];
float yi_dc[1];
float zi_dc[1];
float dir_dc[1];
float esp_dc[1];
unsigned int grid_size_dc[1];
unsigned int max_temp_dc[1];

#include "CUDAMCFLio.cu"
#include "CUDAMCFLmem.cu"
#include "CUDAMCFLrng.cu"
#include "CUDAMCFLtransport.cu"

#include "oracle_api.h"

namespace {

typedef void (*kernel_fn)(MemStruct);

/* One <<<NUM_BLOCKS, NUM_THREADS_PER_BLOCK>>> launch over virtual threads. */
void launch(kernel_fn k, const MemStruct &mem, int nthreads) {
  if (nthreads <= 1) {
    for (unsigned bx = 0; bx < NUM_BLOCKS; ++bx)
      for (unsigned tx = 0; tx < NUM_THREADS_PER_BLOCK; ++tx) {
        blockIdx.x = bx;
        threadIdx.x = tx;
        k(mem);
      }
    return;
  }
  std::vector<std::thread> pool;
  for (int w = 0; w < nthreads; ++w)
    pool.emplace_back([&, w] {
      for (unsigned bx = (unsigned)w; bx < NUM_BLOCKS; bx += (unsigned)nthreads)
        for (unsigned tx = 0; tx < NUM_THREADS_PER_BLOCK; ++tx) {
          blockIdx.x = bx;
          threadIdx.x = tx;
          k(mem);
        }
    });
  for (auto &t : pool) t.join();
}

/* Relaunch until every virtual thread is inactive (CUDAMCFLmain.cu:117-165,
 * 229-273).  Returns the number of relaunches, or -1 past the cap. */
long run_until_done(SimulationStruct *sim, MemStruct &dev, MemStruct &host, int nthreads, long cap) {
  launch(LaunchPhoton_Global, dev, nthreads);
  long i = 0;
  unsigned int active = 1;
  while (active > 0) {
    ++i;
    launch(sim->bulk_method == 1 ? MCd : MCd3D, dev, nthreads);
    memcpy(host.thread_active, dev.thread_active, NUM_THREADS * sizeof(unsigned int));
    active = 0;
    for (unsigned ii = 0; ii < NUM_THREADS; ++ii) active += host.thread_active[ii];
    memcpy(host.num_terminated_photons, dev.num_terminated_photons, sizeof(unsigned long long));
    if (cap > 0 && i > cap) return -1;
  }
  return i;
}

} // namespace

/* CUDAMCFLmain.cu:60-193 without the printing and the file writing. */
static unsigned long long do_one_simulation(SimulationStruct *simulation, unsigned long long *x, unsigned int *a,
                                            double *tempfhd, unsigned long long *rd, unsigned long long *tt,
                                            unsigned long long *fhd_raw, int nthreads,
                                            unsigned long long *time_xyt = nullptr) {
  MemStruct DeviceMem, HostMem;
  const int num_x = (int)(4 * (simulation->esp) * (float)simulation->grid_size);
  const int num_y = (int)(4 * (simulation->esp) * (float)simulation->grid_size);
  const int num_z = (int)((simulation->esp) * (float)simulation->grid_size);
  const int fhd_size = num_x * num_y * num_z;
  const int xy_size = simulation->det.nx + simulation->det.ny * simulation->det.nx;
  HostMem.x = x;
  HostMem.a = a;
  InitMemStructs(&HostMem, &DeviceMem, simulation);
  InitDCMem(simulation);
  if (simulation->do_temp_sim == 1) {
    const int nxt = simulation->det.x_temp_numdets, nyt = simulation->det.y_temp_numdets;
    for (int xi = 0; xi < nxt; xi++)
      HostMem.tdet_pos_x[xi] = xi * simulation->det.x_temp_sepdets -
                               ((nxt - 1) * simulation->det.x_temp_sepdets) / 2 + simulation->det.x0_temp_det;
    for (int yi = 0; yi < nyt; yi++)
      HostMem.tdet_pos_y[yi] = yi * simulation->det.y_temp_sepdets -
                               ((nyt - 1) * simulation->det.y_temp_sepdets) / 2 + simulation->det.y0_temp_det;
    memcpy(DeviceMem.tdet_pos_x, HostMem.tdet_pos_x, nxt * sizeof(float));
    memcpy(DeviceMem.tdet_pos_y, HostMem.tdet_pos_y, nyt * sizeof(float));
  }
  run_until_done(simulation, DeviceMem, HostMem, nthreads, 0);
  CopyDeviceToHostMem(&HostMem, &DeviceMem, simulation);
  unsigned long long photons_finished = *HostMem.num_terminated_photons;
  for (int xyz = 0; xyz < fhd_size; xyz++)
    tempfhd[xyz] = ((double)HostMem.fhd[xyz] / (0xFFFFFFFF * photons_finished));
  if (rd) memcpy(rd, HostMem.Rd_xy, xy_size * sizeof(unsigned long long));
  if (tt) memcpy(tt, HostMem.Tt_xy, xy_size * sizeof(unsigned long long));
  if (fhd_raw) memcpy(fhd_raw, HostMem.fhd, (size_t)fhd_size * sizeof(unsigned long long));
  if (time_xyt)
    memcpy(time_xyt, HostMem.time_xyt, (size_t)simulation->det.x_temp_numdets * simulation->det.y_temp_numdets *
                                           simulation->det.temp_bins * sizeof(unsigned long long));
  FreeMemStructs(&HostMem, &DeviceMem);
  return photons_finished;
}

/* CUDAMCFLmain.cu:196-288. */
static unsigned long long do_one_simulation_fl(SimulationStruct *simulation, unsigned long long *x, unsigned int *a,
                                               unsigned long long *tempvoxelR, unsigned long long *tempvoxelT,
                                               int nthreads) {
  MemStruct DeviceMem, HostMem;
  const int xy_size = simulation->det.nx + simulation->det.ny * simulation->det.nx;
  HostMem.x = x;
  HostMem.a = a;
  InitMemStructs(&HostMem, &DeviceMem, simulation);
  InitDCMem(simulation);
  if (run_until_done(simulation, DeviceMem, HostMem, nthreads, 10000) < 0) return 0;
  CopyDeviceToHostMem(&HostMem, &DeviceMem, simulation);
  for (int ijk = 0; ijk < xy_size; ijk++) {
    tempvoxelR[ijk] = HostMem.Rd_xy[ijk];
    tempvoxelT[ijk] = HostMem.Tt_xy[ijk];
  }
  unsigned long long photons_finished = *HostMem.num_terminated_photons;
  FreeMemStructs(&HostMem, &DeviceMem);
  return photons_finished;
}

/* read_simulation_data leaves the table of the other bulk method as a
 * one-entry dummy with an uninitialised count (CUDAMCFLio.cu:519-524,642-644)
 * and InitDCMem then uploads count+2 entries of it (CUDAMCFLmem.cu:84,87).
 * On a GPU that copy reads past the dummy or fails; the transport of that
 * method never reads the table.  Give the unused table a zeroed, correctly
 * sized allocation so that the host build stays in bounds. */
static void normalise_unused_tables(SimulationStruct *sim) {
  if (sim->bulk_method == 2) {
    free(sim->layers);
    sim->n_layers = 0;
    sim->layers = (LayerStruct *)calloc(2, sizeof(LayerStruct));
  } else {
    free(sim->bulks);
    sim->n_bulks = 0;
    sim->bulks = (BulkStruct *)calloc(2, sizeof(BulkStruct));
  }
}

extern "C" int ref_run_mci(const char *mci_path, const char *safeprimes_path, unsigned long long seed_exc,
                           unsigned long long seed_fl, int nthreads, int write_files, oracle_result *res) {
  SimulationStruct *simulations = NULL;
  memset(res, 0, sizeof(*res));
  int n_sim = read_simulation_data((char *)mci_path, &simulations, 0);
  if (n_sim == 0) return -1;
  SimulationStruct *sim = &simulations[0];
  normalise_unused_tables(sim);
  std::vector<unsigned long long> x(NUM_THREADS);
  std::vector<unsigned int> a(NUM_THREADS);
  if (init_RNG(x.data(), a.data(), NUM_THREADS, safeprimes_path, seed_exc)) return -2;

  const int num_x = (int)(4 * (sim->esp) * sim->grid_size);
  const int num_y = (int)(4 * (sim->esp) * sim->grid_size);
  const int num_z = (int)((sim->esp) * sim->grid_size);
  const int fhd_size = num_x * num_y * num_z;
  const int nx2 = sim->det.nx, ny2 = sim->det.ny;
  const int xy_size = nx2 + ny2 * nx2;
  res->grid[0] = num_x; res->grid[1] = num_y; res->grid[2] = num_z;
  res->image[0] = nx2; res->image[1] = ny2;
  res->Rd = (unsigned long long *)calloc(xy_size, 8);
  res->Tt = (unsigned long long *)calloc(xy_size, 8);
  res->fhd = (unsigned long long *)calloc(fhd_size > 0 ? fhd_size : 1, 8);
  res->flR = (double *)calloc(xy_size, 8);
  res->flT = (double *)calloc(xy_size, 8);
  std::vector<double> Fx(fhd_size > 0 ? fhd_size : 1);

  if (sim->do_temp_sim == 1) {
    res->time_size = (long)sim->det.x_temp_numdets * sim->det.y_temp_numdets * (long)sim->det.temp_bins;
    res->time_xyt = (unsigned long long *)calloc(res->time_size > 0 ? res->time_size : 1, 8);
  }
  res->photons_exc = do_one_simulation(sim, x.data(), a.data(), Fx.data(), res->Rd, res->Tt, res->fhd, nthreads,
                                       res->time_xyt);
  res->number_of_photons = sim->number_of_photons;
  if (write_files) {
    /* Write_Simulation_Results needs a MemStruct holding the host tallies. */
    MemStruct hm;
    memset(&hm, 0, sizeof(hm));
    hm.Rd_xy = res->Rd;
    hm.Tt_xy = res->Tt;
    std::vector<float> tpx(sim->det.x_temp_numdets + 1), tpy(sim->det.y_temp_numdets + 1);
    if (sim->do_temp_sim == 1) {
      const int nxt = sim->det.x_temp_numdets, nyt = sim->det.y_temp_numdets;
      for (int xi = 0; xi < nxt; xi++)
        tpx[xi] = xi * sim->det.x_temp_sepdets - ((nxt - 1) * sim->det.x_temp_sepdets) / 2 + sim->det.x0_temp_det;
      for (int yi = 0; yi < nyt; yi++)
        tpy[yi] = yi * sim->det.y_temp_sepdets - ((nyt - 1) * sim->det.y_temp_sepdets) / 2 + sim->det.y0_temp_det;
      hm.tdet_pos_x = tpx.data();
      hm.tdet_pos_y = tpy.data();
      hm.time_xyt = res->time_xyt;
    }
    Write_Simulation_Results(&hm, sim, 0);
    /* the reference leaves <out>_time.dat open (CUDAMCFLio.cu:168-187); its
     * process exit flushes it, this driver does it here */
    fflush(NULL);
    if (sim->fhd_activated == 1) oracle_write_phd(sim->outp_filename, Fx.data(), num_x, num_y, num_z);
  }

  if (init_RNG(x.data(), a.data(), NUM_THREADS, safeprimes_path, seed_fl)) return -2;
  if (sim->do_fl_sim != 0) {
    const double dx = sim->det.dx, dy = sim->det.dy;
    for (int n = 0; n < (int)sim->n_layers + 2; n++) sim->layers[n].mua = sim->layers[n].muaf;
    for (int n = 0; n < (int)sim->n_bulks + 2; n++) sim->bulks[n].mua = sim->bulks[n].muaf;
    sim->number_of_photons = (unsigned long long)sim->number_of_photons_per_voxel;
    sim->dir = 0.0f;
    sim->fhd_activated = 0;
    std::vector<unsigned long long> tR(xy_size), tT(xy_size);
    for (int ix = 0; ix < num_x; ix++)
      for (int iy = 0; iy < num_y; iy++)
        for (int iz = 0; iz < num_z; iz++) {
          int index = ix + num_x * (iy + iz * num_y);
          short bd = sim->bulk_info[index];
          float xi = ((float)ix / sim->grid_size) - 2 * sim->esp;
          float yi = ((float)iy / sim->grid_size) - 2 * sim->esp;
          float zi = ((float)iz / sim->grid_size);
          sim->xi = xi; sim->yi = yi; sim->zi = zi;
          std::fill(tR.begin(), tR.end(), 0ull);
          std::fill(tT.begin(), tT.end(), 0ull);
          unsigned long long voxel_status = 1;
          double voxelw = 0;
          if (sim->bulk_method == 2) {
            if (sim->bulks[bd].albedof < 1) {
              voxel_status = do_one_simulation_fl(sim, x.data(), a.data(), tR.data(), tT.data(), nthreads);
              voxelw = ((double)sim->bulks[bd].eY * (double)(1 - sim->bulks[bd].albedof) * Fx[index]) /
                       (double)(voxel_status * 0xFFFFFFFF);
              res->fl_voxels += 1;
            }
          }
          /* bulk method 1 never simulates emission: its gate albedof < 0 is
           * never true (CUDAMCFLmain.cu:520,535; CUDAMCFLio.cu:460,500). */
          if (voxel_status == 0) res->failed_voxels += 1;
          if (sim->bulk_method == 2 && sim->bulks[bd].albedof < 1) res->photons_fl += voxel_status;
          for (int ij = 0; ij < xy_size; ij++) {
            double tempvwR = voxelw * (double)tR[ij];
            double tempvwT = voxelw * (double)tT[ij];
            if (res->flR[ij] + tempvwR < DBL_MAX) res->flR[ij] += tempvwR / (dx * dy);
            if (res->flT[ij] + tempvwT < DBL_MAX) res->flT[ij] += tempvwT / (dx * dy);
          }
        }
    if (write_files) oracle_write_fl_images(sim->outp_filename, res->flR, res->flT, nx2, ny2);
  }
  FreeSimulationStruct(simulations, n_sim);
  return 0;
}

/* The reference's own parser (CUDAMCFLio.cu:243-659), flattened. */
extern "C" int ref_parse_mci(const char *mci_path, oracle_sim *out) {
  SimulationStruct *simulations = NULL;
  memset(out, 0, sizeof(*out));
  int n_sim = read_simulation_data((char *)mci_path, &simulations, 0);
  if (n_sim == 0) return -1;
  SimulationStruct *sim = &simulations[0];
  out->number_of_photons = sim->number_of_photons;
  out->number_of_photons_per_voxel = sim->number_of_photons_per_voxel;
  out->n_bulks = sim->n_bulks;
  out->start_weight = sim->start_weight;
  out->grid_size = sim->grid_size;
  out->esp = sim->esp;
  out->xi = sim->xi; out->yi = sim->yi; out->zi = sim->zi; out->dir = sim->dir;
  out->fhd_activated = sim->fhd_activated;
  out->do_fl_sim = sim->do_fl_sim;
  out->bulk_method = sim->bulk_method;
  out->det_dx = sim->det.dx; out->det_dy = sim->det.dy;
  out->det_nx = sim->det.nx; out->det_ny = sim->det.ny;
  out->det_x0 = sim->det.x0; out->det_y0 = sim->det.y0;
  out->do_temp_sim = sim->do_temp_sim;
  out->tdet_x0 = sim->det.x0_temp_det; out->tdet_y0 = sim->det.y0_temp_det;
  out->tdet_nx = (int)sim->det.x_temp_numdets; out->tdet_ny = (int)sim->det.y_temp_numdets;
  out->tdet_sep_x = sim->det.x_temp_sepdets; out->tdet_sep_y = sim->det.y_temp_sepdets;
  out->tdet_r = sim->det.temp_det_r;
  out->tdet_face = (int)sim->det.temp_rort;
  out->tdet_bins = (long)sim->det.temp_bins;
  out->tdet_max = (unsigned long long)sim->det.max_temp;
  if (sim->bulk_method == 1) {
    if (sim->n_layers > ORACLE_MAX_LAYERS) return -3;
    out->n_layers = (int)sim->n_layers;
    for (unsigned i = 0; i < sim->n_layers + 2; ++i) {
      const LayerStruct &L = sim->layers[i];
      /* the parser sets only n of the outer media; the rest is uninitialised */
      if (i == 0 || i == sim->n_layers + 1) {
        out->layers[i] = oracle_layer{0, 0, 0, 0, 0, L.n, 0, 0, 0, 0};
        continue;
      }
      out->layers[i] = oracle_layer{L.z_min, L.z_max, L.mutr, L.mua, L.g, L.n, L.flc, L.muaf, L.eY, L.albedof};
    }
    const IncStruct &I = sim->inclusion;
    out->inclusion = oracle_inclusion{I.x, I.y, I.z, I.r, I.mutr, I.mua, I.g, I.n, I.flc, I.muaf, I.eY, I.albedof};
  }
  if (sim->bulk_method == 2) {
    if (sim->n_bulks > ORACLE_MAX_BULKS) return -3;
    for (unsigned i = 0; i < sim->n_bulks + 2; ++i) {
      const BulkStruct &b = sim->bulks[i];
      out->bulks[i] = oracle_bulk{b.mutr, b.mua, b.g, b.n, b.flc, b.muaf, b.eY, b.albedof, 0.0f};
    }
    const int num_x = (int)(4 * sim->esp * sim->grid_size);
    const int num_y = (int)(4 * sim->esp * sim->grid_size);
    const int num_z = (int)(sim->esp * sim->grid_size);
    size_t n = (size_t)num_x * num_y * num_z;
    short *lab = (short *)malloc(n * sizeof(short) + 2);
    memcpy(lab, sim->bulk_info, n * sizeof(short));
    out->bulk_info = lab;
  }
  FreeSimulationStruct(simulations, n_sim);
  return 0;
}

/* The reference's own init_RNG (CUDAMCFLrng.cu:31-90). */
extern "C" int ref_init_rng(unsigned long long *x, unsigned int *a, unsigned int n, const char *path,
                            unsigned long long seed) {
  return init_RNG(x, a, n, path, seed);
}
