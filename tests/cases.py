"""Small reference-expressible test media (cubic voxels of 1/grid cm, lateral
extent 4*esp, labels 0-9) shared by the oracle and the GPU tests."""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

import cudamcfl_gb300 as mc
from oracle import pyoracle


@dataclass
class Case:
    name: str
    esp: float
    grid: int
    labels: np.ndarray       # (nz, ny, nx) uint8
    columns: list            # .mci columns per label 1..n: (n, mua, mus, flc, AbsCExi, AbsCEmi, eY, g)
    n_out: float
    photons: int
    per_voxel: int
    det: tuple               # dx, dy, nx, ny, x0, y0
    source: tuple = (0.0, 0.0, 0.0)
    do_fl: int = 1
    # time-resolved detectors: (x0, y0, nx, ny, sep_x, sep_y, radius, face, bins, max_fs) or None
    temporal: tuple | None = None
    # 1: voxel-boundary stepping in both the oracle and the engine
    exact_stepping: int = 0
    # optional per-voxel emission-strength factor (nz, ny, nx) float32, in both engines
    fluor_map: np.ndarray | None = None

    @property
    def dims(self):
        n = int(round(4 * self.esp * self.grid))
        return n, n, int(round(self.esp * self.grid))

    def bulks(self):
        b = [mc.outer_bulk(self.n_out)]
        b += [mc.bulk_from_mci_columns(*c) for c in self.columns]
        b.append(mc.outer_bulk(self.n_out))
        return b

    def start_weight(self) -> int:
        n1 = np.float64(np.float32(self.n_out))
        n2 = np.float64(np.float32(self.columns[0][0]))
        r = (n1 - n2) / (n1 + n2)
        return int(np.float64(0xFFFFFFFF) * (1 - r * r))

    def oracle_sim(self):
        """oracle_sim with the same floats as the engine medium."""
        s = pyoracle.CSim()
        s.bulk_method = 2
        s.number_of_photons = self.photons
        s.number_of_photons_per_voxel = self.per_voxel
        s.grid_size = self.grid
        s.esp = self.esp
        s.do_fl_sim = self.do_fl
        s.fhd_activated = 1 if self.do_fl in (1, 2) else 0
        s.det_dx, s.det_dy, s.det_nx, s.det_ny, s.det_x0, s.det_y0 = self.det
        s.xi, s.yi, s.zi = self.source
        s.dir = 1.0
        bl = self.bulks()
        s.n_bulks = len(bl) - 2
        for i, b in enumerate(bl):
            s.bulks[i] = pyoracle.CBulk(b.mutr, b.mua, b.g, b.n, b.flc, b.muaf, b.eY, b.albedof, b.mus)
        s.start_weight = self.start_weight()
        lab = np.ascontiguousarray(self.labels.astype(np.int16))
        s.bulk_info = lab.ctypes.data_as(pyoracle.ctypes.POINTER(pyoracle.ctypes.c_short))
        s._keep = [lab]
        if self.fluor_map is not None:
            fm = np.ascontiguousarray(self.fluor_map, dtype=np.float32)
            s.fluor_map = fm.ctypes.data_as(pyoracle.ctypes.POINTER(pyoracle.ctypes.c_float))
            s._keep.append(fm)
        s.exact_stepping = self.exact_stepping
        if self.temporal:
            x0, y0, tnx, tny, sx, sy, r, face, bins, tmax = self.temporal
            s.do_temp_sim = 1
            s.tdet_x0, s.tdet_y0, s.tdet_nx, s.tdet_ny = x0, y0, tnx, tny
            s.tdet_sep_x, s.tdet_sep_y, s.tdet_r, s.tdet_face = sx, sy, r, face
            s.tdet_bins, s.tdet_max = bins, tmax
        return s

    def engine_medium(self, ctx):
        nx, ny, nz = self.dims
        e = np.float32(self.esp)
        return ctx.medium(self.labels, self.bulks(), vox_per_cm=(float(self.grid),) * 3,
                          half_x=float(np.float32(2) * e), half_y=float(np.float32(2) * e), thickness=float(e),
                          fluor_map=self.fluor_map)

    def run_desc(self, seed_exc, seed_fl, photons=None):
        dx, dy, nx, ny, x0, y0 = self.det
        return mc.run_desc(photons or self.photons, source=self.source, det=mc.Detector(x0, y0, dx, dy, nx, ny),
                           photons_per_voxel=self.per_voxel if self.do_fl else 0,
                           fluence=1 if self.do_fl in (1, 2) else 0, seed_exc=seed_exc, seed_fl=seed_fl,
                           start_weight=self.start_weight(), tdet=self.temporal,
                           exact_stepping=self.exact_stepping)

    def write_mci(self, d: str) -> str:
        """Writes <d>/<name>.mci and its bulk file in the reference's grammar."""
        nx, ny, nz = self.dims
        bulk = os.path.join(d, self.name + ".bulk")
        with open(bulk, "w") as f:
            f.write(" ".join(str(int(v)) for v in self.labels.ravel()) + "\n")
        dx, dy, dnx, dny, x0, y0 = self.det
        lines = ["# test medium " + self.name, "1.0 # file version", "1 # runs", "2 # method",
                 f"{self.name}-out A", f"{self.photons} # photons", f"{self.per_voxel} # photons per voxel",
                 f"{self.grid} # grid", f"{self.do_fl} # fluorescence", f"{dx} {dy}", f"{dnx} {dny}", f"{x0} {y0}",
                 "{} {} {}".format(*self.source)]
        if self.temporal:
            x0, y0, tnx, tny, sx, sy, r, face, bins, tmax = self.temporal
            lines += ["1 # temporal", f"{x0} {y0}", f"{tnx} {tny}", f"{sx} {sy}", f"{r}", f"{face}", f"{bins}",
                      f"{tmax}"]
        else:
            lines += ["0 # temporal", "0 0", "1 1", "1 1", "0.5", "0", "10", "1000"]
        lines += [f"{len(self.columns)} # bulks", f"{self.esp} # thickness", f"{self.n_out}"]
        for c in self.columns:
            lines.append(" ".join(repr(float(v)) for v in c))
        lines += [f"{self.n_out}", os.path.basename(bulk)]
        path = os.path.join(d, self.name + ".mci")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        return path


def nearest_emitters(labels, bulks, voxel_cm, point, k):
    """Linear indices (x fastest) of the k voxels of fluorescent labels
    (albedof < 1) whose centres lie nearest to point (x, y, z in cm; the grid
    is centred on x = y = 0 and starts at z = 0), nearest first."""
    nz, ny, nx = labels.shape
    fluorescent = np.array([b.albedof < 1 for b in bulks])
    iz, iy, ix = np.nonzero(fluorescent[labels])
    x = (ix + 0.5) * voxel_cm[0] - nx * voxel_cm[0] / 2
    y = (iy + 0.5) * voxel_cm[1] - ny * voxel_cm[1] / 2
    z = (iz + 0.5) * voxel_cm[2]
    d = (x - point[0]) ** 2 + (y - point[1]) ** 2 + (z - point[2]) ** 2
    order = np.argsort(d, kind="stable")[:k]
    return (ix + nx * (iy + ny * iz))[order]


def emitter_map(shape, voxels, values=None):
    """A fluorophore map that is zero except at the given linear voxel
    indices (1 there, or the given values): the emission phase then runs
    exactly those voxels, in both engines, while the excitation medium is
    unchanged (the map scales only the emission weights)."""
    m = np.zeros(shape, dtype=np.float32)
    m.ravel()[voxels] = 1.0 if values is None else values
    return m


def config1_parity(photons=1_250_000, per_voxel=33000, emitters=6) -> Case:
    """The reference-expressible variant of the config-1 sphere medium: esp
    = 2, grid_size = 25, i.e. 200 x 200 x 50 voxels of 0.04 cm over 8 x 8 x 2
    cm (the reference fixes the lateral extent to 4 esp and cubic voxels);
    background n 1.4 in air, mu_a 0.1, mu_s 100, g 0.9; a fluorescent sphere
    r = 0.25 cm at the slab centre (fluorophore absorption 0.05/cm at both
    wavelengths, quantum yield 0.1; the reference keeps mu_s at emission);
    Gaussian beam at the top centre; 100 x 100 images of 0.04 cm.  The
    emission phase runs the `emitters` sphere voxels nearest the top of the
    sphere (a fluorophore map of ones there, zero elsewhere), since the
    reference's schedule costs at least 32768 photons per voxel."""
    esp, grid = 2.0, 25
    lab = _labels(esp, grid)
    nz, ny, nx = lab.shape
    z = (np.arange(nz) + 0.5) / grid
    y = (np.arange(ny) + 0.5) / grid - 2 * esp
    x = (np.arange(nx) + 0.5) / grid - 2 * esp
    m = (x[None, None, :] ** 2 + y[None, :, None] ** 2 + (z[:, None, None] - 1.0) ** 2) <= 0.25 ** 2
    lab[m] = 2
    c = Case("config1_parity", esp, grid, lab,
             [(1.4, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.4, 0.1, 100.0, 1.0, 0.05, 0.05, 0.1, 0.9)],
             1.0, photons, per_voxel, (0.04, 0.04, 100, 100, 0.0, 0.0))
    v = nearest_emitters(lab, c.bulks(), (1 / grid,) * 3, (0.0, 0.0, 0.75), emitters)
    c.fluor_map = emitter_map(lab.shape, v)
    return c


def _labels(esp, grid, fill=1):
    n = int(round(4 * esp * grid))
    return np.full((int(round(esp * grid)), n, n), fill, dtype=np.uint8)


def tiny(photons=40000, per_voxel=40000) -> Case:
    lab = _labels(0.5, 4)
    lab[0, 3:5, 3:5] = 2
    return Case("tiny", 0.5, 4, lab,
                [(1.4, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.4, 0.1, 100.0, 1.0, 0.05, 0.02, 0.1, 0.9)],
                1.0, photons, per_voxel, (0.1, 0.1, 20, 20, 0.0, 0.0))


def mismatch(photons=40000, per_voxel=40000) -> Case:
    """Internal index mismatch (Fresnel and total internal reflection at
    label changes), absorbing inclusion, off-centre beam and detector."""
    lab = _labels(0.5, 6)
    nz, ny, nx = lab.shape
    lab[1:, 4:8, 5:9] = 2
    lab[0, 8:10, 2:5] = 3
    return Case("mismatch", 0.5, 6, lab,
                [(1.37, 0.2, 60.0, 0.0, 0.0, 0.0, 0.0, 0.8), (1.52, 0.5, 40.0, 2.0, 0.1, 0.04, 0.2, 0.7),
                 (1.33, 1.0, 80.0, 0.5, 0.2, 0.1, 0.05, 0.0)],
                1.0, photons, per_voxel, (0.08, 0.07, 24, 20, 0.1, -0.05), (0.13, -0.07, 0.0))


def glass(photons=40000, per_voxel=40000) -> Case:
    """A scattering-free label (mus = 0) crossed by the beam: the half-voxel
    march and sphere back-projection of MoveToFirstBoundary."""
    lab = _labels(0.5, 4)
    lab[0, 3:5, 3:5] = 2
    lab[1, 2:6, 2:6] = 3
    return Case("glass", 0.5, 4, lab,
                [(1.4, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.4, 0.05, 0.0, 0.0, 0.0, 0.0, 0.0, 0.9),
                 (1.4, 0.2, 90.0, 1.0, 0.05, 0.02, 0.1, 0.85)],
                1.0, photons, per_voxel, (0.1, 0.1, 20, 20, 0.0, 0.0))


def sphere(photons=40000, per_voxel=33000) -> Case:
    """Config-1-like: a fluorescent sphere r=0.25 under a centred beam."""
    esp, grid = 1.0, 10
    lab = _labels(esp, grid)
    nz, ny, nx = lab.shape
    z = (np.arange(nz) + 0.5) / grid
    y = (np.arange(ny) + 0.5) / grid - 2 * esp
    x = (np.arange(nx) + 0.5) / grid - 2 * esp
    m = (x[None, None, :] ** 2 + y[None, :, None] ** 2 + (z[:, None, None] - 0.5) ** 2) <= 0.25 ** 2
    lab[m] = 2
    return Case("sphere", esp, grid, lab,
                [(1.4, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.4, 0.1, 100.0, 1.0, 0.05, 0.05, 0.1, 0.9)],
                1.0, photons, per_voxel, (0.04, 0.04, 50, 50, 0.0, 0.0))


def deep(photons=40000, per_voxel=40000) -> Case:
    """tiny with the fluorescent block one voxel layer below the beam entry
    (0.25-0.5 cm deep), away from the voxels whose photon hitting density the
    reference's first-photon random-number reuse touches."""
    lab = _labels(0.5, 4)
    lab[1, 3:5, 3:5] = 2
    return Case("deep", 0.5, 4, lab,
                [(1.4, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.4, 0.1, 100.0, 1.0, 0.05, 0.02, 0.1, 0.9)],
                1.0, photons, per_voxel, (0.1, 0.1, 20, 20, 0.0, 0.0))


def blocks(photons=40000, per_voxel=2000) -> Case:
    """A larger grid (80 x 80 x 20 voxels of 0.05 cm) with long homogeneous
    runs: a block of another refractive index and a fluorescent sphere in a
    weakly scattering background (mean free path about one voxel), so that
    voxel-boundary stepping crosses many faces and free cubes of radius up to
    9 voxels."""
    esp, grid = 1.0, 20
    lab = _labels(esp, grid)
    nz, ny, nx = lab.shape
    lab[4:12, 30:44, 20:36] = 3
    z = (np.arange(nz) + 0.5) / grid
    y = (np.arange(ny) + 0.5) / grid - 2 * esp
    x = (np.arange(nx) + 0.5) / grid - 2 * esp
    m = ((x[None, None, :] - 0.4) ** 2 + (y[None, :, None] + 0.3) ** 2 + (z[:, None, None] - 0.45) ** 2) <= 0.3 ** 2
    lab[m] = 2
    return Case("blocks", esp, grid, lab,
                [(1.4, 0.1, 20.0, 0.0, 0.0, 0.0, 0.0, 0.8), (1.4, 0.1, 20.0, 1.0, 0.5, 0.2, 0.1, 0.8),
                 (1.6, 0.3, 40.0, 0.0, 0.0, 0.0, 0.0, 0.7)],
                1.0, photons, per_voxel, (0.05, 0.05, 60, 60, 0.0, 0.0))


def sparse(photons=40000, per_voxel=2000) -> Case:
    """A weakly scattering slab (mean free path 2 mm, 0.5 cm thick) on a grid
    of 8 x 8 x 2 voxels of 0.25 cm: photons leave the grid's lateral extent
    often, so voxel-boundary stepping walks the medium of label 1 beyond it,
    and come back through its lateral faces into a block of another index."""
    lab = _labels(0.5, 4)
    lab[1, 2:6, 2:6] = 2
    lab[0, 3:5, 0:2] = 3
    return Case("sparse", 0.5, 4, lab,
                [(1.4, 0.2, 5.0, 0.0, 0.0, 0.0, 0.0, 0.9), (1.5, 0.2, 5.0, 1.0, 0.5, 0.2, 0.1, 0.8),
                 (1.3, 0.5, 8.0, 0.0, 0.0, 0.0, 0.0, 0.7)],
                1.0, photons, per_voxel, (0.1, 0.1, 30, 30, 0.0, 0.0))


def sparse_offset(photons=40000, per_voxel=2000) -> Case:
    """sparse with the beam 0.5 cm beyond the grid's lateral extent: every
    photon starts in the medium of label 1 outside the grid."""
    c = sparse(photons, per_voxel)
    c.name = "sparse_offset"
    c.source = (1.5, 0.25, 0.0)
    return c


def timed(photons=40000, per_voxel=40000, face=0, base=None) -> Case:
    """mismatch (or another case) with a 3 x 2 array of time-resolved
    detectors, discs of 0.15 cm 0.25 cm apart, on the entry (face 0) or exit
    face (1): 40 bins over 0.15 ns (entry) or 0.3 ns (exit)."""
    c = (base or mismatch)(photons, per_voxel)
    c.name = c.name + ("_timed" if face == 0 else "_timed_exit")
    c.temporal = (0.1, -0.05, 3, 2, 0.25, 0.25, 0.15, face, 40, 150000 if face == 0 else 300000)
    return c


def mismatch_timed(photons=40000, per_voxel=40000) -> Case:
    return timed(photons, per_voxel, 0, mismatch)


def glass_timed_exit(photons=40000, per_voxel=40000) -> Case:
    return timed(photons, per_voxel, 1, glass)


def exact(base):
    """A case with voxel-boundary stepping in both the oracle and the engine."""
    def make(photons=40000, per_voxel=40000) -> Case:
        c = base(photons, per_voxel)
        c.name = c.name + "_exact"
        c.exact_stepping = 1
        return c
    return make


ALL = {"tiny": tiny, "mismatch": mismatch, "glass": glass, "sphere": sphere, "mismatch_timed": mismatch_timed,
       "glass_timed_exit": glass_timed_exit}


@dataclass
class LayeredCase:
    """A layered medium with one spherical inclusion (the reference's bulk
    method 1), excitation only."""
    name: str
    grid: int
    slabs: list              # per slab: (n, mua, mus, flc, AbsCExi, AbsCEmi, eY, g, thickness)
    n_up: float
    n_down: float
    inclusion: tuple         # (x, y, z, r, n, mua, mus, flc, AbsCExi, AbsCEmi, eY, g)
    photons: int
    det: tuple               # dx, dy, nx, ny, x0, y0
    source: tuple = (0.0, 0.0, 0.0)
    do_fl: int = 2           # photon hitting density on (the reference runs no emission for layers)
    temporal: tuple | None = None
    per_voxel: int = 40000

    def layers(self):
        return mc.layers_from_mci_columns(self.n_up, self.slabs, self.n_down)

    def incl(self):
        return mc.inclusion_from_mci_columns(*self.inclusion)

    def start_weight(self) -> int:
        n1 = np.float64(np.float32(self.n_up))
        n2 = np.float64(np.float32(self.slabs[0][0]))
        r = (n1 - n2) / (n1 + n2)
        return int(np.float64(0xFFFFFFFF) * (1 - r * r))

    def oracle_sim(self):
        s = pyoracle.CSim()
        s.bulk_method = 1
        s.number_of_photons = self.photons
        s.number_of_photons_per_voxel = self.per_voxel
        s.grid_size = self.grid
        lay = self.layers()
        s.esp = lay[-2].z_max
        s.do_fl_sim = self.do_fl
        s.fhd_activated = 1 if self.do_fl in (1, 2) else 0
        s.det_dx, s.det_dy, s.det_nx, s.det_ny, s.det_x0, s.det_y0 = self.det
        s.xi, s.yi, s.zi = self.source
        s.dir = 1.0
        s.n_bulks = 0
        s.start_weight = self.start_weight()
        s.n_layers = len(lay) - 2
        for i, L in enumerate(lay):
            s.layers[i] = pyoracle.CLayer(*(getattr(L, f) for f, _ in L._fields_))
        c = self.incl()
        s.inclusion = pyoracle.CInclusion(*(getattr(c, f) for f, _ in c._fields_))
        if self.temporal:
            x0, y0, tnx, tny, sx, sy, r, face, bins, tmax = self.temporal
            s.do_temp_sim = 1
            s.tdet_x0, s.tdet_y0, s.tdet_nx, s.tdet_ny = x0, y0, tnx, tny
            s.tdet_sep_x, s.tdet_sep_y, s.tdet_r, s.tdet_face = sx, sy, r, face
            s.tdet_bins, s.tdet_max = bins, tmax
        return s

    def engine_medium(self, ctx):
        return ctx.medium_layered(self.layers(), self.incl(), self.grid)

    def run_desc(self, seed_exc, seed_fl, photons=None):
        dx, dy, nx, ny, x0, y0 = self.det
        return mc.run_desc(photons or self.photons, source=self.source, det=mc.Detector(x0, y0, dx, dy, nx, ny),
                           fluence=1 if self.do_fl in (1, 2) else 0, seed_exc=seed_exc, seed_fl=seed_fl,
                           start_weight=self.start_weight(), tdet=self.temporal)

    def write_mci(self, d: str) -> str:
        dx, dy, dnx, dny, x0, y0 = self.det
        lines = ["# layered test medium " + self.name, "1.0 # file version", "1 # runs", "1 # method",
                 f"{self.name}-out A", f"{self.photons} # photons", f"{self.per_voxel} # photons per voxel",
                 f"{self.grid} # grid", f"{self.do_fl} # fluorescence", f"{dx} {dy}", f"{dnx} {dny}", f"{x0} {y0}",
                 "{} {} {}".format(*self.source)]
        if self.temporal:
            x0t, y0t, tnx, tny, sx, sy, r, face, bins, tmax = self.temporal
            lines += ["1 # temporal", f"{x0t} {y0t}", f"{tnx} {tny}", f"{sx} {sy}", f"{r}", f"{face}", f"{bins}",
                      f"{tmax}"]
        else:
            lines += ["0 # temporal", "0 0", "1 1", "1 1", "0.5", "0", "10", "1000"]
        lines += [f"{len(self.slabs)} # layers", f"{self.n_up}"]
        lines += [" ".join(repr(float(v)) for v in sl) for sl in self.slabs]
        lines += [f"{self.n_down}", " ".join(repr(float(v)) for v in self.inclusion)]
        path = os.path.join(d, self.name + ".mci")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        return path


def layered(photons=40000, per_voxel=40000) -> LayeredCase:
    """Two slabs with an index step between them, an absorbing inclusion
    across the interface, off-centre beam."""
    return LayeredCase("layered", 10,
                       [(1.4, 0.1, 90.0, 0.0, 0.0, 0.0, 0.0, 0.9, 0.3),
                        (1.33, 0.3, 60.0, 0.0, 0.0, 0.0, 0.0, 0.8, 0.5)],
                       1.0, 1.0, (0.1, -0.05, 0.35, 0.2, 1.4, 0.8, 70.0, 0.0, 0.0, 0.0, 0.0, 0.85),
                       photons, (0.05, 0.05, 40, 40, 0.0, 0.0), (0.05, 0.02, 0.0), per_voxel=per_voxel)


def layered_timed_exit(photons=40000, per_voxel=40000) -> LayeredCase:
    """layered with a scattering-free inclusion and time-resolved detectors
    on the exit face."""
    c = layered(photons, per_voxel)
    c.name = "layered_timed_exit"
    c.inclusion = (0.0, 0.0, 0.5, 0.15, 1.5, 0.05, 0.0, 0.0, 0.0, 0.0, 0.0, 0.9)
    c.temporal = (0.0, 0.0, 2, 2, 0.3, 0.3, 0.2, 1, 30, 300000)
    return c


LAYERED = {"layered": layered, "layered_timed_exit": layered_timed_exit}

# voxel-boundary stepping
EXACT = {n + "_exact": exact(f) for n, f in {"tiny": tiny, "mismatch": mismatch, "glass": glass, "sphere": sphere,
                                              "deep": deep, "blocks": blocks, "sparse": sparse,
                                              "sparse_offset": sparse_offset, "mismatch_timed": mismatch_timed,
                                              "glass_timed_exit": glass_timed_exit}.items()}
