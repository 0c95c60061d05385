"""Seeded synthetic media in the bulk-descriptor format.

Bulk-descriptor matrices as the reference's medium notebook builds them
(Bulk_descriptor_creator.ipynb: spheres and cylinders burned into a
background label, written x fastest), generated with numpy from a seed so the
benchmarks and tests need no input files.  Labels are uint8 arrays of shape
(nz, ny, nx); optical properties follow the .mci columns
(n mua mus flc AbsCExi AbsCEmi eY g) and are turned into the reference's
derived quantities by :func:`cudamcfl_gb300.bulk_from_mci_columns`.

Workloads (all cm):
  config1   slab 4 x 4 x 2 in 50^3 voxels, n=1.4 in air, mua 0.1, mus 100,
            g 0.9; one fluorescent sphere r=0.25 at the centre (fluorophore
            absorption 0.05, quantum yield 0.1); Gaussian beam at the top
            centre; 100 x 100 images of 0.04.
  config2   200 x 200 x 100 voxels of 0.02; 8 labels with mua U(0.02, 0.5),
            mus U(50, 150), g U(0.8, 0.95), n=1.4; 5-20 spheres
            (r 0.1-0.5) and cylinders (r 0.05-0.3, random axis) carrying a
            U(0, 1) fluorophore map; quantum yield U(0.05, 0.2).
  config5   the large precision-study medium: 512 x 512 x 256 voxels of
            0.01 cm, mu_s' = 20/cm, fp32 fluorophore map, wide-field source.
  raster    the 16 x 16 grid of beam positions over the top face used for the
            batched sweep, with log-uniform budgets.
Emission scattering equals excitation scattering: the reference's emission
phase keeps the excitation 1/(mua+mus) (CUDAMCFLmain.cu:458-461).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import Bulk, Detector, bulk_from_mci_columns, outer_bulk


@dataclass
class SyntheticMedium:
    labels: np.ndarray              # uint8 (nz, ny, nx)
    bulks: list                     # n+2 Bulk entries
    voxel_cm: tuple                 # (dx, dy, dz)
    fluor_map: np.ndarray | None = None
    det: Detector | None = None
    source: tuple = (0.0, 0.0, 0.0)
    info: dict = field(default_factory=dict)

    @property
    def shape(self):
        return self.labels.shape

    @property
    def nvox(self) -> int:
        return int(self.labels.size)


def _grid_centres(shape, voxel_cm):
    nz, ny, nx = shape
    dx, dy, dz = voxel_cm
    x = (np.arange(nx) + 0.5) * dx - nx * dx / 2
    y = (np.arange(ny) + 0.5) * dy - ny * dy / 2
    z = (np.arange(nz) + 0.5) * dz
    return z[:, None, None], y[None, :, None], x[None, None, :]


def _box(shape, voxel_cm, lo, hi):
    """Index slices of the voxels whose centres may lie in [lo, hi] (cm,
    x/y/z), widened by one voxel; the mask is then evaluated on that box only,
    with the same centre coordinates as on the whole grid."""
    nz, ny, nx = shape
    sl = []
    for n, d, a, b, off in ((nz, voxel_cm[2], lo[2], hi[2], 0.0), (ny, voxel_cm[1], lo[1], hi[1], ny * voxel_cm[1] / 2),
                            (nx, voxel_cm[0], lo[0], hi[0], nx * voxel_cm[0] / 2)):
        i0 = int(np.floor((a + off) / d)) - 1
        i1 = int(np.ceil((b + off) / d)) + 1
        sl.append(slice(min(max(i0, 0), n), min(max(i1, 0), n)))
    return tuple(sl)


def _centres_in(shape, voxel_cm, box):
    z, y, x = _grid_centres(shape, voxel_cm)
    return z[box[0], :, :], y[:, box[1], :], x[:, :, box[2]]


def add_sphere(labels, voxel_cm, centre, r, label, fmap=None, fval=None):
    box = _box(labels.shape, voxel_cm, [c - r for c in centre], [c + r for c in centre])
    z, y, x = _centres_in(labels.shape, voxel_cm, box)
    m = (x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2 <= r * r
    labels[box][m] = label
    if fmap is not None:
        fmap[box][m] = fval if np.isscalar(fval) else fval[box][m]
    return int(m.sum())


def add_cylinder(labels, voxel_cm, point, axis, r, half_len, label, fmap=None, fval=None):
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    ext = [abs(a[i]) * half_len + r for i in range(3)]
    box = _box(labels.shape, voxel_cm, [point[i] - ext[i] for i in range(3)], [point[i] + ext[i] for i in range(3)])
    z, y, x = _centres_in(labels.shape, voxel_cm, box)
    px, py, pz = x - point[0], y - point[1], z - point[2]
    t = px * a[0] + py * a[1] + pz * a[2]
    d2 = px * px + py * py + pz * pz - t * t
    m = (d2 <= r * r) & (np.abs(t) <= half_len)
    labels[box][m] = label
    if fmap is not None:
        fmap[box][m] = fval if np.isscalar(fval) else fval[box][m]
    return int(m.sum())


def config1(n_inside: float = 1.4, n_outside: float = 1.0) -> SyntheticMedium:
    nx = ny = nz = 50
    vox = (0.08, 0.08, 0.04)
    lab = np.ones((nz, ny, nx), dtype=np.uint8)
    nin = add_sphere(lab, vox, (0.0, 0.0, 1.0), 0.25, 2)
    bulks = [outer_bulk(n_outside),
             bulk_from_mci_columns(n_inside, 0.1, 100.0, 0.0, 0.0, 0.0, 0.0, 0.9),
             bulk_from_mci_columns(n_inside, 0.1, 100.0, 1.0, 0.05, 0.05, 0.1, 0.9),
             outer_bulk(n_outside)]
    det = Detector(0.0, 0.0, 0.04, 0.04, 100, 100)
    return SyntheticMedium(lab, bulks, vox, None, det, (0.0, 0.0, 0.0), {"sphere_voxels": nin})


def config2(seed: int = 2, n_labels: int = 8) -> SyntheticMedium:
    rng = np.random.default_rng(seed)
    nx, ny, nz = 200, 200, 100
    vox = (0.02, 0.02, 0.02)
    lab = np.ones((nz, ny, nx), dtype=np.uint8)
    fmap = np.zeros((nz, ny, nx), dtype=np.float32)
    mua = rng.uniform(0.02, 0.5, n_labels)
    mus = rng.uniform(50.0, 150.0, n_labels)
    g = rng.uniform(0.8, 0.95, n_labels)
    qy = rng.uniform(0.05, 0.2, n_labels)
    fl_abs = rng.uniform(0.01, 0.1, n_labels)  # fluorophore absorption at excitation [1/cm]
    fl_emi = rng.uniform(0.005, 0.05, n_labels)
    bulks = [outer_bulk(1.0)]
    for i in range(n_labels):
        fluorescent = i > 0
        bulks.append(bulk_from_mci_columns(1.4, mua[i], mus[i], 1.0 if fluorescent else 0.0,
                                           fl_abs[i] if fluorescent else 0.0, fl_emi[i] if fluorescent else 0.0,
                                           qy[i] if fluorescent else 0.0, g[i]))
    bulks.append(outer_bulk(1.0))
    n_inc = int(rng.integers(5, 21))
    shapes = []
    fval = rng.uniform(0.0, 1.0, size=lab.shape).astype(np.float32)
    for _ in range(n_inc):
        label = int(rng.integers(2, n_labels + 1))
        c = (rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5), rng.uniform(0.3, 1.7))
        if rng.uniform() < 0.5:
            r = rng.uniform(0.1, 0.5)
            nvx = add_sphere(lab, vox, c, r, label, fmap, fval)
            shapes.append(("sphere", label, r, nvx))
        else:
            r = rng.uniform(0.05, 0.3)
            ax = rng.normal(size=3)
            nvx = add_cylinder(lab, vox, c, ax, r, rng.uniform(0.3, 1.5), label, fmap, fval)
            shapes.append(("cylinder", label, r, nvx))
    det = Detector(0.0, 0.0, 0.04, 0.04, 100, 100)
    return SyntheticMedium(lab, bulks, vox, fmap, det, (0.0, 0.0, 0.0), {"inclusions": shapes})


def config5(seed: int = 5, shape=(256, 512, 512), voxel: float = 0.01, n_labels: int = 8,
            musp: float = 20.0) -> SyntheticMedium:
    """The large precision-study medium: (nz, ny, nx) = 256 x 512 x 512
    voxels of 0.01 cm (5.12 x 5.12 x 2.56 cm) with a fp32 U(0, 1) fluorophore
    map (268 MB), reduced scattering mu_s' = mu_s (1 - g) = 20/cm in every
    label, mua U(0.02, 0.5), g U(0.8, 0.95), n = 1.4, 5-20 spheres and
    cylinders as in config2; a uniform wide-field source covers the top face
    and the R/T images are 256 x 256 pixels over the same area.
    config5(shape=(64, 128, 128), voxel=0.04) is the same medium at a quarter
    of the resolution (the size a CPU oracle finishes)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    vox = (voxel, voxel, voxel)
    lab = np.ones((nz, ny, nx), dtype=np.uint8)
    fmap = np.zeros((nz, ny, nx), dtype=np.float32)
    mua = rng.uniform(0.02, 0.5, n_labels)
    g = rng.uniform(0.8, 0.95, n_labels)
    mus = musp / (1.0 - g)
    qy = rng.uniform(0.05, 0.2, n_labels)
    fl_abs = rng.uniform(0.01, 0.1, n_labels)
    fl_emi = rng.uniform(0.005, 0.05, n_labels)
    bulks = [outer_bulk(1.0)]
    for i in range(n_labels):
        fluorescent = i > 0
        bulks.append(bulk_from_mci_columns(1.4, mua[i], mus[i], 1.0 if fluorescent else 0.0,
                                           fl_abs[i] if fluorescent else 0.0, fl_emi[i] if fluorescent else 0.0,
                                           qy[i] if fluorescent else 0.0, g[i]))
    bulks.append(outer_bulk(1.0))
    hx, hy, depth = nx * voxel / 2, ny * voxel / 2, nz * voxel
    fval = rng.random(size=lab.shape, dtype=np.float32)
    shapes = []
    for _ in range(int(rng.integers(5, 21))):
        label = int(rng.integers(2, n_labels + 1))
        c = (rng.uniform(-hx + 0.5, hx - 0.5), rng.uniform(-hy + 0.5, hy - 0.5), rng.uniform(0.3, depth - 0.3))
        if rng.uniform() < 0.5:
            r = rng.uniform(0.1, 0.5)
            shapes.append(("sphere", label, r, add_sphere(lab, vox, c, r, label, fmap, fval)))
        else:
            r = rng.uniform(0.05, 0.3)
            ax = rng.normal(size=3)
            shapes.append(("cylinder", label, r,
                           add_cylinder(lab, vox, c, ax, r, rng.uniform(0.3, 1.5), label, fmap, fval)))
    det = Detector(0.0, 0.0, 2 * hx / 256, 2 * hy / 256, 256, 256)
    return SyntheticMedium(lab, bulks, vox, fmap, det, (0.0, 0.0, 0.0),
                           {"inclusions": shapes, "widefield": (2 * hx, 2 * hy), "musp": musp})


def raster_sources(n: int = 16, extent: float = 4.0, seed: int = 3, lo: float = 1e6, hi: float = 5e7,
                   scale: float = 1.0):
    """n x n beam positions over a square of side extent centred on 0, and a
    log-uniform photon budget per position (multiplied by scale)."""
    rng = np.random.default_rng(seed)
    step = extent / n
    xs = -extent / 2 + step * (np.arange(n) + 0.5)
    pos = [(float(x), float(y)) for y in xs for x in xs]
    budgets = np.exp(rng.uniform(np.log(lo), np.log(hi), n * n)) * scale
    return pos, [max(1, int(b)) for b in budgets]
