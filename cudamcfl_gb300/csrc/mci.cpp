/*
 * The reference's file surface, kept as a drop-in:
 *   - the .mci grammar and the bulk-descriptor matrix (read_simulation_data,
 *     readfloats, readints, CUDAMCFLio.cu:193-659);
 *   - the command-line arguments (interpret_arg, CUDAMCFLio.cu:30-55);
 *   - init_RNG over a multiplier file (CUDAMCFLrng.cu:31-90);
 *   - the output files _param.dat, _Trans.dat, _Refl.dat
 *     (Write_Simulation_Results, CUDAMCFLio.cu:57-191), _PHD-Ascii.dat
 *     (CUDAMCFLmain.cu:368-392), _FlR.dat and _FlT.dat
 *     (CUDAMCFLmain.cu:604-647);
 *   - DoOneSimulation, DoOneSimulationFl and main (CUDAMCFLmain.cu:60-668)
 *     on top of the engine.
 *
 * The parser reads numbers with the same scanf conversions and line buffers
 * (200 characters for float lines, 500 otherwise) as the reference, so the
 * parsed values are the same floats.  Differences, each an error where the
 * reference would read uninitialised or out-of-range memory: a bulk file
 * with fewer labels than the grid, or a label outside 0..n_bulks+1, is a
 * parse error; a grid whose 4*esp*grid_size is not an integer is rejected
 * (the reference sizes its arrays by truncation and indexes them by
 * rounding, CUDAMCFLio.cu:609 vs CUDAMCFLtransport.cu:255).  The photon-count
 * clamps of the reference are kept (CUDAMCFLio.cu:312-315,321-324).
 */
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "mcfl_internal.h"

using namespace mcfl;

namespace {

constexpr unsigned kRefThreads = 32768; /* NUM_THREADS, CUDAMCFL.h:18-20 */
constexpr int kNFloats = 12, kNInts = 5;

/* Line of up to n floats; lines without a leading number are skipped. */
bool read_floats(int n, float *t, FILE *f) {
  char line[200];
  int got = 0;
  if (n > kNFloats) return false;
  while (got <= 0) {
    if (feof(f)) return false;
    if (!fgets(line, sizeof(line), f)) line[0] = 0;
    std::memset(t, 0, kNFloats * sizeof(float));
    got = sscanf(line, "%f %f %f %f %f %f %f %f %f %f %f %f", &t[0], &t[1], &t[2], &t[3], &t[4], &t[5], &t[6], &t[7],
                 &t[8], &t[9], &t[10], &t[11]);
    if (got > n) return false;
  }
  return true;
}

bool read_ints(int n, int *t, FILE *f) {
  char line[MCFL_STR_LEN];
  int got = 0;
  if (n > kNInts) return false;
  while (got <= 0) {
    if (feof(f)) return false;
    if (!fgets(line, sizeof(line), f)) line[0] = 0;
    std::memset(t, 0, kNInts * sizeof(int));
    got = sscanf(line, "%d %d %d %d %d", &t[0], &t[1], &t[2], &t[3], &t[4]);
    if (got > n) return false;
  }
  return true;
}

bool is_letter(char a) { return (a >= 'A' && a <= 'Z') || (a >= 'a' && a <= 'z'); }

int parse_error(FILE *f, const char *what) {
  if (f) fclose(f);
  fail(MCFL_E_PARSE, what);
  return 0;
}

void set_bulk(mcfl_bulk &b, const float *t) {
  b.n = t[0];
  b.mua = t[1] + t[3] * t[4];
  b.muaf = t[1] + t[3] * t[5];
  b.eY = t[6];
  b.flc = t[3];
  b.g = t[7];
  b.mutr = t[2] == 0.0f ? FLT_MAX : 1.0f / (t[1] + t[2]);
  b.albedof = t[2] / (t[3] * t[4] + t[2]);
  b.mus = t[2];
}

void set_outer(mcfl_bulk &b, float n) {
  b = mcfl_bulk{FLT_MAX, 0.0f, 1.0f, n, 0.0f, 0.0f, 0.0f, 0.0f};
}

/* Bulk matrix: every non-blank character c is the label c - '0'
 * (CUDAMCFLio.cu:618-636). */
int read_bulk_file(mcfl_simulation &s, long long expected) {
  std::ifstream in(s.bulkinfo_filename);
  if (!in) return fail(MCFL_E_IO, std::string("cannot open bulk file ") + s.bulkinfo_filename);
  s.bulk_info = (unsigned char *)calloc((size_t)expected + 1, 1);
  if (!s.bulk_info) return fail(MCFL_E_NOMEM, "bulk matrix allocation");
  long long count = 0;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream iss(line);
    char ch;
    while (iss >> ch) {
      const int v = ch - '0';
      if (count < expected) {
        if (v < 0 || v > (int)s.n_bulks + 1)
          return fail(MCFL_E_PARSE, "bulk file: label outside 0..n_bulks+1 at value " + std::to_string(count));
        s.bulk_info[count] = (unsigned char)v;
      }
      ++count;
    }
  }
  s.bulk_values_read = count;
  if (count < expected)
    return fail(MCFL_E_PARSE, "bulk file holds " + std::to_string(count) + " labels, grid needs " +
                                  std::to_string(expected));
  return MCFL_OK;
}

} // namespace

namespace mcfl {
void simulation_geometry(const mcfl_simulation *sim, float *half_x, float *half_y, float *esp, float *g) {
  *half_x = 2 * sim->esp;
  *half_y = 2 * sim->esp;
  *esp = sim->esp;
  *g = (float)sim->grid_size;
}
} // namespace mcfl

extern "C" int mcfl_read_simulation_data(const char *filename, mcfl_simulation **simulations, int ignoreAdetection) {
  (void)ignoreAdetection; /* the reference accepts and ignores it */
  if (!filename || !simulations) return parse_error(nullptr, "null argument");
  *simulations = nullptr;
  FILE *f = fopen(filename, "r");
  if (!f) {
    fail(MCFL_E_IO, std::string("cannot open ") + filename);
    return 0;
  }
  float ft[kNFloats];
  int it[kNInts];
  if (!read_floats(1, ft, f)) return parse_error(f, "file version");
  if (!read_ints(1, it, f)) return parse_error(f, "number of runs");
  const int n_sim = it[0];
  if (n_sim <= 0 || n_sim > 1000) return parse_error(f, "number of runs");
  mcfl_simulation *sims = (mcfl_simulation *)calloc((size_t)n_sim, sizeof(mcfl_simulation));
  if (!sims) return parse_error(f, "allocation");
  *simulations = sims;
  for (int i = 0; i < n_sim; ++i) {
    mcfl_simulation &s = sims[i];
    std::strncpy(s.inp_filename, filename, MCFL_STR_LEN - 1);
    if (!read_ints(1, it, f)) return parse_error(f, "bulk description method");
    s.bulk_method = it[0];
    /* output file name and A/B flag; the name must start with a letter */
    {
      int got = 0;
      char line[MCFL_STR_LEN], str[MCFL_STR_LEN];
      char aorb = 0;
      while (got <= 0) {
        s.begin = ftell(f);
        if (!fgets(line, sizeof(line), f)) line[0] = 0;
        got = sscanf(line, "%499s %c", str, &aorb);
        if (feof(f) || got > 2) return parse_error(f, "output filename");
        if (got > 0) got = is_letter(str[0]);
      }
      std::strncpy(s.outp_filename, str, MCFL_STR_LEN - 1);
      s.AorB = aorb;
    }
    {
      int got = 0;
      char line[MCFL_STR_LEN];
      unsigned long long nph = 0;
      while (got <= 0) {
        if (!fgets(line, sizeof(line), f)) line[0] = 0;
        nph = 0;
        got = sscanf(line, "%llu", &nph);
        if (feof(f) || got > 1) return parse_error(f, "number of photons");
      }
      if (nph <= kRefThreads) nph = kRefThreads - 1;
      s.number_of_photons = nph;
    }
    if (!read_ints(1, it, f)) return parse_error(f, "photons per voxel");
    s.number_of_photons_per_voxel = it[0] <= (int)kRefThreads ? kRefThreads - 1 : (unsigned)it[0];
    if (!read_ints(1, it, f)) return parse_error(f, "grid size");
    s.grid_size = it[0];
    if (!read_ints(1, it, f)) return parse_error(f, "fluorescence flag");
    s.do_fl_sim = it[0];
    s.fhd_activated = (it[0] == 1 || it[0] == 2) ? 1 : 0;
    if (it[0] < 0 || it[0] > 2) return parse_error(f, "fluorescence flag");
    if (!read_floats(2, ft, f)) return parse_error(f, "image dx dy");
    s.det.dx = ft[0];
    s.det.dy = ft[1];
    if (!read_ints(2, it, f)) return parse_error(f, "image nx ny");
    s.det.nx = it[0];
    s.det.ny = it[1];
    if (!read_floats(2, ft, f)) return parse_error(f, "image x0 y0");
    s.det.x0 = ft[0];
    s.det.y0 = ft[1];
    if (!read_floats(3, ft, f)) return parse_error(f, "source position");
    s.xi = ft[0];
    s.yi = ft[1];
    s.zi = ft[2];
    if (!read_ints(1, it, f)) return parse_error(f, "temporal flag");
    s.do_temp_sim = it[0];
    if (it[0] != 0 && it[0] != 1) return parse_error(f, "temporal flag");
    if (!read_floats(2, ft, f)) return parse_error(f, "temporal detector centre");
    s.det.x0_temp_det = ft[0];
    s.det.y0_temp_det = ft[1];
    if (!read_ints(2, it, f)) return parse_error(f, "temporal detector count");
    s.det.x_temp_numdets = (unsigned)it[0];
    s.det.y_temp_numdets = (unsigned)it[1];
    if (!read_floats(2, ft, f)) return parse_error(f, "temporal detector separation");
    s.det.x_temp_sepdets = ft[0];
    s.det.y_temp_sepdets = ft[1];
    if (!read_floats(1, ft, f)) return parse_error(f, "temporal detector radius");
    s.det.temp_det_r = ft[0];
    if (!read_ints(1, it, f)) return parse_error(f, "temporal detector location");
    s.det.temp_rort = (unsigned)it[0];
    if (it[0] != 0 && it[0] != 1) return parse_error(f, "temporal detector location");
    if (!read_ints(1, it, f)) return parse_error(f, "temporal bins");
    s.det.temp_bins = (unsigned long)it[0];
    if (!read_ints(1, it, f)) return parse_error(f, "max time");
    s.det.max_temp = (unsigned long)it[0];
    double n1 = 1, n2 = 1;
    if (s.bulk_method == 1) {
      if (!read_ints(1, it, f)) return parse_error(f, "number of layers");
      if (it[0] < 1 || it[0] > 98) return parse_error(f, "number of layers");
      s.n_layers = (unsigned)it[0];
      s.layers = (mcfl_layer *)calloc(s.n_layers + 2, sizeof(mcfl_layer));
      s.bulks = (mcfl_bulk *)calloc(2, sizeof(mcfl_bulk));
      if (!read_floats(1, ft, f)) return parse_error(f, "upper refractive index");
      s.layers[0].n = ft[0];
      float dtot = 0;
      for (unsigned l = 1; l <= s.n_layers; ++l) {
        if (!read_floats(9, ft, f)) return parse_error(f, "layer data");
        mcfl_layer &L = s.layers[l];
        L.n = ft[0];
        L.mua = ft[1] + ft[3] * ft[4];
        L.muaf = ft[1] + ft[3] * ft[5];
        L.eY = ft[6];
        L.flc = ft[3];
        L.g = ft[7];
        L.z_min = dtot;
        dtot += ft[8];
        L.z_max = dtot;
        L.mutr = ft[2] == 0.0f ? FLT_MAX : 1.0f / (ft[1] + ft[2]);
        L.albedof = ft[2] / (ft[3] * ft[4] + ft[2]);
      }
      s.esp = dtot;
      if (!read_floats(1, ft, f)) return parse_error(f, "lower refractive index");
      s.layers[s.n_layers + 1].n = ft[0];
      if (!read_floats(12, ft, f)) return parse_error(f, "inclusion data");
      mcfl_inclusion &I = s.inclusion;
      I.x = ft[0]; I.y = ft[1]; I.z = ft[2]; I.r = ft[3]; I.n = ft[4];
      I.mua = ft[5] + ft[7] * ft[8];
      I.muaf = ft[5] + ft[7] * ft[9];
      I.flc = ft[7];
      I.eY = ft[10];
      I.g = ft[11];
      I.mutr = ft[6] == 0.0f ? FLT_MAX : 1.0f / (ft[5] + ft[6]);
      I.albedof = ft[6] / (ft[7] * ft[8] + ft[6]);
      n1 = s.layers[0].n;
      n2 = s.layers[1].n;
      /* the photon-hitting-density grid main sizes for either method
       * (CUDAMCFLmain.cu:340-342) */
      const float g = (float)s.grid_size;
      s.num_x = (int)(4 * s.esp * g);
      s.num_y = (int)(4 * s.esp * g);
      s.num_z = (int)(s.esp * g);
    } else if (s.bulk_method == 2) {
      if (!read_ints(1, it, f)) return parse_error(f, "number of bulk descriptors");
      if (it[0] < 1 || it[0] > MCFL_MAX_BULKS) return parse_error(f, "number of bulk descriptors");
      s.n_bulks = (unsigned)it[0];
      s.bulks = (mcfl_bulk *)calloc(s.n_bulks + 2, sizeof(mcfl_bulk));
      s.layers = (mcfl_layer *)calloc(2, sizeof(mcfl_layer));
      if (!read_floats(1, ft, f)) return parse_error(f, "bulk thickness");
      s.esp = ft[0];
      if (!read_floats(1, ft, f)) return parse_error(f, "outer refractive index");
      set_outer(s.bulks[0], ft[0]);
      for (unsigned b = 1; b <= s.n_bulks; ++b) {
        if (!read_floats(8, ft, f)) return parse_error(f, "bulk descriptor data");
        set_bulk(s.bulks[b], ft);
      }
      if (!read_floats(1, ft, f)) return parse_error(f, "lower refractive index");
      set_outer(s.bulks[s.n_bulks + 1], ft[0]);
      {
        int got = 0;
        char line[MCFL_STR_LEN], str[MCFL_STR_LEN];
        while (got <= 0) {
          if (feof(f)) return parse_error(f, "bulk matrix filename");
          if (!fgets(line, sizeof(line), f)) line[0] = 0;
          got = sscanf(line, "%499s", str);
        }
        std::strncpy(s.bulkinfo_filename, str, MCFL_STR_LEN - 1);
      }
      const float g = (float)s.grid_size;
      s.num_x = (int)(4 * s.esp * g);
      s.num_y = (int)(4 * s.esp * g);
      s.num_z = (int)(s.esp * g);
      const float nxr = nearbyintf(4 * s.esp * g);
      if ((float)s.num_x != nxr || s.num_x <= 0 || s.num_z <= 0)
        return parse_error(f, "4*thickness*grid_size must be a positive integer");
      if (read_bulk_file(s, (long long)s.num_x * s.num_y * s.num_z) != MCFL_OK) {
        fclose(f);
        return 0;
      }
      n1 = s.bulks[0].n;
      n2 = s.bulks[1].n;
    } else {
      return parse_error(f, "bulk description method must be 1 or 2");
    }
    double r = (n1 - n2) / (n1 + n2);
    r = r * r;
    s.start_weight = (unsigned int)((double)0xFFFFFFFF * (1 - r));
    s.dir = 1.0f;
    s.end = ftell(f);
  }
  fclose(f);
  return n_sim;
}

extern "C" void mcfl_free_simulation_struct(mcfl_simulation *sims, int n) {
  if (!sims) return;
  for (int i = 0; i < n; ++i) {
    free(sims[i].layers);
    free(sims[i].bulks);
    free(sims[i].bulk_info);
  }
  free(sims);
}

extern "C" int mcfl_interpret_arg(int argc, char *argv[], unsigned long long *seed, int *ignoreAdetection) {
  for (int i = 2; i < argc; i++) {
    int unknown = 1;
    if (!std::strcmp(argv[i], "-A")) {
      unknown = 0;
      if (ignoreAdetection) *ignoreAdetection = 1;
    }
    if (!std::strncmp(argv[i], "-S", 2) && sscanf(argv[i], "%*2c %llu", seed)) unknown = 0;
    if (unknown) {
      fail(MCFL_E_ARG, std::string("unknown argument ") + argv[i]);
      return 1;
    }
  }
  return 0;
}

extern "C" int mcfl_init_RNG(unsigned long long *x, unsigned int *a, unsigned int n_rng, const char *safeprimes_file,
                             unsigned long long xinit) {
  const char *path = (safeprimes_file && *safeprimes_file) ? safeprimes_file : "safeprimes_base32.txt";
  FILE *fp = fopen(path, "r");
  if (!fp) {
    fail(MCFL_E_IO, std::string("cannot open ") + path);
    return 1;
  }
  unsigned int begin = 0, fora, t1, t2;
  if (fscanf(fp, "%u %u %u", &begin, &t1, &t2) != 3) {
    fclose(fp);
    fail(MCFL_E_PARSE, "multiplier file");
    return 1;
  }
  if ((xinit == 0ull) | (((unsigned int)(xinit >> 32)) >= (begin - 1)) | (((unsigned int)xinit) >= 0xfffffffful)) {
    fclose(fp);
    fail(MCFL_E_ARG, "invalid seed");
    return 1;
  }
  for (unsigned int i = 0; i < n_rng; i++) {
    if (fscanf(fp, "%u %u %u", &fora, &t1, &t2) != 3) {
      fclose(fp);
      fail(MCFL_E_PARSE, "multiplier file too short");
      return 1;
    }
    a[i] = fora;
    x[i] = 0;
    while ((x[i] == 0) | (((unsigned int)(x[i] >> 32)) >= (fora - 1)) | (((unsigned int)x[i]) >= 0xfffffffful)) {
      xinit = (xinit & 0xffffffffull) * (begin) + (xinit >> 32);
      x[i] = (unsigned int)floor((((double)((unsigned int)xinit)) / (double)0x100000000) * fora);
      x[i] = x[i] << 32;
      xinit = (xinit & 0xffffffffull) * (begin) + (xinit >> 32);
      x[i] += (unsigned int)xinit;
    }
  }
  fclose(fp);
  return 0;
}

extern "C" int mcfl_write_safeprimes(const char *path, unsigned int count) {
  if (!path || count == 0 || count > 1000000) return fail(MCFL_E_ARG, "mcfl_write_safeprimes: bad argument");
  std::vector<uint32_t> a = count <= kMwcTableEntries + 1
                                ? std::vector<uint32_t>(mwc_table().begin(), mwc_table().begin() + count)
                                : mwc_multipliers(count);
  if (a.size() != count) return fail(MCFL_E_STATE, "not enough multipliers below 2^32");
  FILE *f = fopen(path, "w");
  if (!f) return fail(MCFL_E_IO, std::string("cannot write ") + path);
  for (uint32_t v : a) {
    const uint64_t q = ((uint64_t)v << 31) - 1;
    fprintf(f, "%u %u %u\n", v, (uint32_t)(q >> 32), (uint32_t)q);
  }
  fclose(f);
  return MCFL_OK;
}

/* ---------------------------------------------------------------- writers */

namespace {

std::string out_path(const mcfl_simulation *sim, const char *suffix) { return std::string(sim->outp_filename) + suffix; }

int write_image(const std::string &path, int nx, int ny, const double *img, const unsigned long long *raw,
                double scale) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) return fail(MCFL_E_IO, "cannot write " + path);
  for (int y = 0; y < ny; y++) {
    for (int x = 0; x < nx; x++) fprintf(f, " %E ", img ? img[y * nx + x] : (double)raw[y * nx + x] / scale);
    fprintf(f, " \n ");
  }
  fclose(f);
  return MCFL_OK;
}

} // namespace

extern "C" int mcfl_Write_Simulation_Results(const mcfl_simulation *sim, const unsigned long long *Rd_xy,
                                             const unsigned long long *Tt_xy, double simulation_time_s) {
  if (!sim || !Rd_xy || !Tt_xy) return fail(MCFL_E_ARG, "mcfl_Write_Simulation_Results: null argument");
  const double dx = (double)sim->det.dx, dy = (double)sim->det.dy;
  const double scale1 = (double)0xFFFFFFFF * (double)sim->number_of_photons;
  const double scale2 = scale1 * dx * dy;
  FILE *in = fopen(sim->inp_filename, "r");
  if (!in) return fail(MCFL_E_IO, std::string("cannot open ") + sim->inp_filename);
  const std::string pp = out_path(sim, "_param.dat");
  FILE *pf = fopen(pp.c_str(), "w");
  if (!pf) {
    fclose(in);
    return fail(MCFL_E_IO, "cannot write " + pp);
  }
  fprintf(pf, "Compilation date: %s, %s. \n\n", __DATE__, __TIME__);
  fprintf(pf, "A1 \t# Version number of the file format.\n\n");
  fprintf(pf, "####\n");
  fprintf(pf, "# Data categories include: \n");
  fprintf(pf, "# InParm, RAT, \n");
  fprintf(pf, "# A_l, A_z, Rd_r, Rd_a, Tt_r, Tt_a, \n");
  fprintf(pf, "# A_rz, Rd_ra, Tt_ra \n");
  fprintf(pf, "####\n\n");
  fprintf(pf, "# User time: %.2f sec\n\n", simulation_time_s);
  fprintf(pf, "InParam\t\t# Input parameters:\n");
  fseek(in, sim->begin, SEEK_SET);
  char line[MCFL_STR_LEN];
  while (sim->end > ftell(in)) {
    if (!fgets(line, sizeof(line), in)) break;
    fputs(line, pf);
  }
  fclose(in);
  fclose(pf);
  int rc = write_image(out_path(sim, "_Trans.dat"), sim->det.nx, sim->det.ny, nullptr, Tt_xy, scale2);
  if (rc) return rc;
  return write_image(out_path(sim, "_Refl.dat"), sim->det.nx, sim->det.ny, nullptr, Rd_xy, scale2);
}

namespace mcfl {

void time_positions(const mcfl_time_detectors &td, float *px, float *py) {
  for (int xi = 0; xi < td.nx; xi++) px[xi] = xi * td.sep_x - ((td.nx - 1) * td.sep_x) / 2 + td.x0;
  for (int yi = 0; yi < td.ny; yi++) py[yi] = yi * td.sep_y - ((td.ny - 1) * td.sep_y) / 2 + td.y0;
}

} // namespace mcfl

namespace {

mcfl_time_detectors time_detectors_of(const mcfl_simulation *sim) {
  mcfl_time_detectors td;
  std::memset(&td, 0, sizeof(td));
  if (sim->do_temp_sim != 1) return td;
  td.nx = (int)sim->det.x_temp_numdets;
  td.ny = (int)sim->det.y_temp_numdets;
  td.x0 = sim->det.x0_temp_det;
  td.y0 = sim->det.y0_temp_det;
  td.sep_x = sim->det.x_temp_sepdets;
  td.sep_y = sim->det.y_temp_sepdets;
  td.radius = sim->det.temp_det_r;
  td.face = (int)sim->det.temp_rort;
  td.bins = (int)sim->det.temp_bins;
  td.max_fs = (unsigned long long)sim->det.max_temp;
  return td;
}

} // namespace

extern "C" int mcfl_write_time(const mcfl_simulation *sim, const unsigned long long *time_xyt) {
  if (!sim || !time_xyt) return fail(MCFL_E_ARG, "mcfl_write_time: null argument");
  const mcfl_time_detectors td = time_detectors_of(sim);
  if (td.nx <= 0 || td.ny <= 0 || td.bins <= 0) return fail(MCFL_E_ARG, "mcfl_write_time: no time-resolved detectors");
  std::vector<float> px((size_t)td.nx), py((size_t)td.ny);
  mcfl::time_positions(td, px.data(), py.data());
  const double scale1 = (double)0xFFFFFFFF * (double)sim->number_of_photons;
  const std::string p = out_path(sim, "_time.dat");
  FILE *f = fopen(p.c_str(), "w");
  if (!f) return fail(MCFL_E_IO, "cannot write " + p);
  fprintf(f, "#x y timebins[numbins]\n");
  for (int ix = 0; ix < td.nx; ix++)
    for (int iy = 0; iy < td.ny; iy++) {
      fprintf(f, "%f %f ", px[ix], py[iy]);
      for (int it = 0; it < td.bins; it++)
        fprintf(f, " %E ", (double)time_xyt[ix + (size_t)td.nx * (iy + (size_t)it * td.ny)] / scale1);
      fprintf(f, " \n ");
    }
  fclose(f);
  return MCFL_OK;
}

extern "C" int mcfl_write_phd(const mcfl_simulation *sim, const double *fhd) {
  if (!sim || !fhd) return fail(MCFL_E_ARG, "mcfl_write_phd: null argument");
  const std::string p = out_path(sim, "_PHD-Ascii.dat");
  FILE *f = fopen(p.c_str(), "w");
  if (!f) return fail(MCFL_E_IO, "cannot write " + p);
  fprintf(f, "%llu\t%llu\t%llu\n", (unsigned long long)sim->num_x, (unsigned long long)sim->num_y,
          (unsigned long long)sim->num_z);
  const long long n = (long long)sim->num_x * sim->num_y * sim->num_z;
  for (long long i = 0; i < n; ++i) fprintf(f, "%.10E\n", fhd[i]);
  fclose(f);
  return MCFL_OK;
}

extern "C" int mcfl_write_fl_images(const mcfl_simulation *sim, const double *flR, const double *flT) {
  if (!sim || !flR || !flT) return fail(MCFL_E_ARG, "mcfl_write_fl_images: null argument");
  int rc = write_image(out_path(sim, "_FlR.dat"), sim->det.nx, sim->det.ny, flR, nullptr, 1.0);
  if (rc) return rc;
  return write_image(out_path(sim, "_FlT.dat"), sim->det.nx, sim->det.ny, flT, nullptr, 1.0);
}

/* ------------------------------------------------- engine over a .mci run */

extern "C" int mcfl_medium_from_simulation(mcfl_ctx *ctx, const mcfl_simulation *sim, mcfl_medium **medium) {
  if (!sim) return fail(MCFL_E_ARG, "null simulation");
  if (sim->bulk_method == 1) {
    if (!sim->layers) return fail(MCFL_E_ARG, "bulk method 1 without layers");
    mcfl_layered_desc ld;
    std::memset(&ld, 0, sizeof(ld));
    ld.n_layers = (int)sim->n_layers;
    ld.layers = sim->layers;
    ld.inclusion = sim->inclusion;
    ld.grid_size = sim->grid_size;
    return mcfl_medium_create_layered(ctx, &ld, medium);
  }
  if (sim->bulk_method != 2 || !sim->bulk_info || !sim->bulks)
    return fail(MCFL_E_STATE, "unknown bulk method");
  mcfl_medium_desc d;
  std::memset(&d, 0, sizeof(d));
  d.nx = sim->num_x;
  d.ny = sim->num_y;
  d.nz = sim->num_z;
  float g;
  simulation_geometry(sim, &d.half_x, &d.half_y, &d.thickness, &g);
  d.vox_per_cm[0] = d.vox_per_cm[1] = d.vox_per_cm[2] = g;
  d.labels = sim->bulk_info;
  d.fluor_map = nullptr;
  d.n_bulks = (int)sim->n_bulks;
  d.bulks = sim->bulks;
  return mcfl_medium_create(ctx, &d, medium);
}

extern "C" int mcfl_run_desc_from_simulation(const mcfl_simulation *sim, unsigned long long seed,
                                             mcfl_run_desc *run) {
  if (!sim || !run) return fail(MCFL_E_ARG, "null argument");
  std::memset(run, 0, sizeof(*run));
  run->photons = sim->number_of_photons;
  /* the reference simulates emission for voxelized media only (its gate
   * albedof < 0 never holds for bulk method 1, CUDAMCFLmain.cu:520,535) */
  run->photons_per_voxel = sim->do_fl_sim && sim->bulk_method == 2 ? sim->number_of_photons_per_voxel : 0;
  run->fluence = sim->fhd_activated;
  run->seed_exc = seed;
  run->seed_fl = seed + 1;
  run->start_weight = sim->start_weight;
  run->source.kind = MCFL_SOURCE_GAUSS_BEAM;
  run->source.x = sim->xi;
  run->source.y = sim->yi;
  run->source.z = sim->zi;
  run->det.x0 = sim->det.x0;
  run->det.y0 = sim->det.y0;
  run->det.dx = sim->det.dx;
  run->det.dy = sim->det.dy;
  run->det.nx = sim->det.nx;
  run->det.ny = sim->det.ny;
  run->launch_rng_reuse = 1; /* the reference's statistics, quirk included */
  run->tdet = time_detectors_of(sim);
  return MCFL_OK;
}

namespace {

std::mutex g_default_mu;
mcfl_ctx *g_default = nullptr;

mcfl_ctx *default_ctx() {
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default && mcfl_create(-1, &g_default) != MCFL_OK) g_default = nullptr;
  return g_default;
}

} // namespace

extern "C" unsigned long long mcfl_DoOneSimulation(const mcfl_simulation *sim, unsigned long long seed, double *fhd_out,
                                                   unsigned long long *Rd_out, unsigned long long *Tt_out) {
  mcfl_ctx *c = default_ctx();
  if (!c) return 0;
  if (sim && sim->dir != 1.0f) {
    fail(MCFL_E_ARG, "DoOneSimulation: the excitation source is collimated (dir = 1)");
    return 0;
  }
  mcfl_medium *m = nullptr;
  if (mcfl_medium_from_simulation(c, sim, &m) != MCFL_OK) return 0;
  mcfl_run_desc run;
  mcfl_run_desc_from_simulation(sim, seed, &run);
  run.photons_per_voxel = 0;
  run.fluence = fhd_out ? 1 : sim->fhd_activated;
  mcfl_run_out out;
  std::memset(&out, 0, sizeof(out));
  out.Rd = Rd_out;
  out.Tt = Tt_out;
  out.phd = fhd_out;
  const int rc = mcfl_run(c, m, &run, &out);
  mcfl_medium_free(m);
  return rc == MCFL_OK ? out.stats_exc[MCFL_ST_DONE] : 0ull;
}

extern "C" unsigned long long mcfl_DoOneSimulationFl(const mcfl_simulation *sim, unsigned long long seed,
                                                     unsigned long long *tempvoxelR, unsigned long long *tempvoxelT) {
  mcfl_ctx *c = default_ctx();
  if (!c || !sim) return 0;
  mcfl_medium *m = nullptr;
  /* the caller has already replaced mua by muaf (CUDAMCFLmain.cu:458-461):
   * this routine transports with the mua it is given */
  if (mcfl_medium_from_simulation(c, sim, &m) != MCFL_OK) return 0;
  const float g = (float)sim->grid_size;
  const long ix = lrintf((sim->xi + 2 * sim->esp) * g), iy = lrintf((sim->yi + 2 * sim->esp) * g),
             iz = lrintf(sim->zi * g);
  if (ix < 0 || iy < 0 || iz < 0 || ix >= sim->num_x || iy >= sim->num_y || iz >= sim->num_z) {
    mcfl_medium_free(m);
    fail(MCFL_E_ARG, "DoOneSimulationFl: source outside the grid");
    return 0;
  }
  mcfl_run_desc run;
  mcfl_run_desc_from_simulation(sim, seed, &run);
  run.photons = sim->number_of_photons;
  unsigned long long st[MCFL_NSTATS] = {0};
  const unsigned voxel = (unsigned)(ix + (long)sim->num_x * (iy + (long)sim->num_y * iz));
  const int rc = run_single_voxel_emission(c, m, &run, voxel, tempvoxelR, tempvoxelT, st);
  mcfl_medium_free(m);
  return rc == MCFL_OK ? st[MCFL_ST_DONE] : 0ull;
}

namespace {

/* One simulation of a .mci file: run, then every file the reference writes. */
int run_one_simulation(mcfl_ctx *c, mcfl_simulation *sim, unsigned long long seed) {
  mcfl_medium *m = nullptr;
  int rc = mcfl_medium_from_simulation(c, sim, &m);
  if (rc != MCFL_OK) return rc;
  const size_t xy = (size_t)sim->det.nx + (size_t)sim->det.nx * sim->det.ny;
  const size_t nv = (size_t)sim->num_x * sim->num_y * sim->num_z;
  std::vector<unsigned long long> Rd(xy), Tt(xy);
  std::vector<double> phd(nv), flR(xy), flT(xy);
  std::vector<unsigned long long> tim;
  mcfl_run_desc run;
  mcfl_run_out out;
  std::memset(&out, 0, sizeof(out));
  mcfl_run_desc_from_simulation(sim, seed, &run);
  out.Rd = Rd.data();
  out.Tt = Tt.data();
  out.phd = sim->fhd_activated ? phd.data() : nullptr;
  out.flR = flR.data();
  out.flT = flT.data();
  if (run.tdet.nx > 0) {
    tim.assign((size_t)run.tdet.nx * run.tdet.ny * run.tdet.bins, 0ull);
    out.time_xyt = tim.data();
  }
  const auto t0 = std::chrono::steady_clock::now();
  rc = mcfl_run(c, m, &run, &out);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  mcfl_medium_free(m);
  if (rc == MCFL_OK) rc = mcfl_Write_Simulation_Results(sim, Rd.data(), Tt.data(), secs);
  if (rc == MCFL_OK && !tim.empty()) rc = mcfl_write_time(sim, tim.data());
  if (rc == MCFL_OK && sim->fhd_activated == 1) rc = mcfl_write_phd(sim, phd.data());
  /* a layered medium never emits: its emission images are zeros, as the
   * reference writes them */
  if (rc == MCFL_OK && sim->do_fl_sim != 0) rc = mcfl_write_fl_images(sim, flR.data(), flT.data());
  return rc;
}

} // namespace

extern "C" int mcfl_run_mci(const char *mci_path, unsigned long long seed) {
  mcfl_simulation *sims = nullptr;
  const int n = mcfl_read_simulation_data(mci_path, &sims, 0);
  if (n <= 0) return MCFL_E_PARSE;
  mcfl_ctx *c = default_ctx();
  int rc = c ? MCFL_OK : MCFL_E_CUDA;
  /* every run of the file, each with its own outputs and seeds seed + 2i
   * (the reference parses the runs and simulates only the first,
   * CUDAMCFLio.cu:272-274, CUDAMCFLmain.cu:340-668) */
  for (int i = 0; rc == MCFL_OK && i < n; ++i) rc = run_one_simulation(c, &sims[i], seed + 2ull * (unsigned)i);
  mcfl_free_simulation_struct(sims, n);
  return rc;
}
