"""Seeded synthetic scan inputs written in the reference's own file formats.

The reference ships no datasets or benchmarks, so every workload here is
generated: an input file (keywords of parse.cpp:143-320), an xyz file
(4/5/6-column format of parse.cpp:477-585), a parameter file (atom / harm /
pair_ovwrt lines of parse.cpp:615-684) and, for the external-field workload,
a Gaussian cube file (cube_io.cpp:89-139, voxel counts negative = Angstrom).

Workloads (named by what they are):

* ``graphene_72``      72-C graphene patch, 6x6 hexagonal cells, LJ only,
                       10x10 A at 0.1 A, z 10->6 at 0.1 (101x101x41 points).
* ``cluster_60``       60-atom C/N/O/H planar cluster with charges, LJ for
                       C/N/H, Morse for the tip-O pair, Coulomb on,
                       20x20 A at 0.05 A (401x401x41 points).
* ``slab_2048``        2048-atom periodic slab (4 layers, 40x40x30 A cell),
                       vdw_pbc + rigidgrid + external Hartree potential cube
                       (160x160x120), 512x512x41 points.
* ``molecule_batch``   planar molecules of log-uniform [20, 400] atoms, pixel
                       grids from {64^2, 128^2, 256^2}, LJ + Coulomb.

Every generator takes a seed and scaling knobs so that tests can make small
versions of the same systems.

Tip/dummy encoding (shared by all workloads): the tip is O (eps 0.21
kcal/mol, sigma 3.0 A).  The reference's ``harm k r0`` is an XY spring
(interactions.cpp:252-266) and the vertical tip-dummy length comes from the
dummy-tip LJ minimum sigma_mix * 2^(1/6) (simulation.cpp:218-225).  A spring
of k = 0.5 kcal/mol/A^2 with rest length 4 A is therefore written as
``harm 0.5 0.0`` plus a dummy ``atom X 20.0 4.127``:
(3.0 + 4.127) / 2 * 2^(1/6) = 4.000 A.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# Bohr radius in Angstrom, as the cube reader uses it (cube_io.hpp:17).
BOHR = 0.52917721092

TIP = ("O", 0.21, 3.0)
DUMMY = ("X", 20.0, 4.127)


def _fmt(v: float) -> str:
    """Shortest text that reads back as the same double (sscanf %lf)."""
    return repr(float(v))


@dataclass
class ScanInput:
    """One scan's input set; ``write(folder)`` emits the reference file formats."""

    name: str
    types: list
    pos: np.ndarray                      # (n, 3) Angstrom, as written to the xyz file
    charges: np.ndarray | None = None    # xyz 5th column (None: 4-column file)
    atom_params: dict = field(default_factory=dict)   # type -> (eps, sig, mass, q)
    overwrites: list = field(default_factory=list)    # (t1, t2, 'lj'|'morse', params...)
    harm: tuple = (0.5, 0.0)
    options: dict = field(default_factory=dict)       # input-file keyword -> value text
    cube: dict | None = None             # {'values': (n0,n1,n2), 'voxel': (3,3) A, 'origin': (3,)}
    fixed: np.ndarray | None = None      # xyz 6th column (flexible mode)

    def write(self, folder: str) -> str:
        os.makedirs(folder, exist_ok=True)
        xyz = os.path.join(folder, f"{self.name}.xyz")
        with open(xyz, "w") as f:
            f.write(f"{len(self.types)}\n{self.name}\n")
            for a, t in enumerate(self.types):
                cols = [t] + [_fmt(c) for c in self.pos[a]]
                if self.charges is not None or self.fixed is not None:
                    q = 0.0 if self.charges is None else self.charges[a]
                    cols.append(_fmt(q))
                if self.fixed is not None:
                    cols.append(str(int(self.fixed[a])))
                f.write(" ".join(cols) + "\n")
        par = os.path.join(folder, f"{self.name}.par")
        with open(par, "w") as f:
            f.write("# synthetic parameters: name eps(energy) sig(A) mass(amu) charge(e)\n")
            for t, (eps, sig, mass, q) in self.atom_params.items():
                f.write(f"atom {t} {_fmt(eps)} {_fmt(sig)} {_fmt(mass)} {_fmt(q)}\n")
            for ow in self.overwrites:
                f.write("pair_ovwrt " + " ".join(str(x) if isinstance(x, str) else _fmt(x)
                                                 for x in ow) + "\n")
            f.write(f"harm {_fmt(self.harm[0])} {_fmt(self.harm[1])}\n")
            for line in getattr(self, "extra_param_lines", []):
                f.write(line + "\n")
        opts = dict(self.options)
        opts["xyzfile"] = os.path.basename(xyz)
        opts["paramfile"] = os.path.basename(par)
        if self.cube is not None:
            cube = os.path.join(folder, f"{self.name}.cube")
            write_cube(cube, self.cube["values"], self.cube["voxel"], self.cube["origin"])
            opts["e_potential_file"] = os.path.basename(cube)
        inp = os.path.join(folder, f"{self.name}.scan")
        with open(inp, "w") as f:
            for k, v in opts.items():
                f.write(f"{k} {v}\n")
        return inp


def base_options(**kw) -> dict:
    """Input keywords shared by the workloads (FIRE + midpoint, gzip off)."""
    o = {
        "tipatom": TIP[0], "dummyatom": DUMMY[0], "units": "kcal/mol",
        "minterm": "ef", "etol": "0.01", "ftol": "0.01", "dt": "0.001",
        "maxsteps": "5000", "minimiser": "FIRE", "integrator": "midpoint",
        "coulomb": "off", "rigidgrid": "off", "flexible": "off",
        "area": "10.0 10.0", "zhigh": "10.0", "zlow": "6.0",
        "dx": "0.1", "dy": "0.1", "dz": "0.1", "bufsize": "10000",
        "gzip": "off", "statistics": "on",
    }
    o.update({k: str(v) for k, v in kw.items()})
    return o


def honeycomb(n1: int, n2: int, bond: float) -> np.ndarray:
    """Honeycomb sites of n1 x n2 hexagonal cells (2 atoms per cell), z = 0."""
    a = bond * math.sqrt(3.0)
    a1 = np.array([a, 0.0])
    a2 = np.array([a / 2, a * math.sqrt(3.0) / 2])
    basis = [np.zeros(2), (a1 + a2) / 3.0]
    pts = []
    for i in range(n1):
        for j in range(n2):
            for b in basis:
                pts.append(i * a1 + j * a2 + b)
    p = np.array(pts)
    return np.column_stack([p, np.zeros(len(p))])


def graphene_72(area: float = 10.0, step: float = 0.1, zhigh: float = 10.0,
                zlow: float = 6.0, dz: float = 0.1, **opt) -> ScanInput:
    """6x6 graphene cells, 72 C at z = 0, LJ only (C-C 1.42 A)."""
    pos = honeycomb(6, 6, 1.42)
    params = {"C": (0.086, 3.4, 12.011, 0.0), TIP[0]: (TIP[1], TIP[2], 15.999, 0.0),
              DUMMY[0]: (DUMMY[1], DUMMY[2], 0.0, 0.0)}
    o = base_options(area=f"{area} {area}", dx=step, dy=step, zhigh=zhigh, zlow=zlow, dz=dz)
    o.update({k: str(v) for k, v in opt.items()})
    return ScanInput("graphene_72", ["C"] * len(pos), pos, None, params, [], (0.5, 0.0), o)


def planar_molecule(n_atoms: int, rng: np.random.Generator, n_h: int | None = None,
                    composition=(("C", 0.6), ("N", 0.1), ("O", 0.1), ("H", 0.2)),
                    jitter: float = 0.05, zspread: float = 0.1, qsigma: float = 0.2,
                    bond: float = 1.40):
    """Seeded aromatic-like cluster on jittered honeycomb sites.

    The ``n_atoms`` sites closest to the centre of a large honeycomb are kept;
    hydrogens take the outermost sites, the other types are shuffled over the
    inner ones.  Charges are N(0, qsigma) shifted to sum to zero.
    """
    cells = int(math.ceil(math.sqrt(n_atoms))) + 4
    sites = honeycomb(cells, cells, bond)[:, :2]
    sites -= sites.mean(axis=0)
    order = np.argsort(np.hypot(sites[:, 0], sites[:, 1]), kind="stable")
    sites = sites[order[:n_atoms]]
    counts = {}
    left = n_atoms
    for t, frac in composition[:-1]:
        counts[t] = int(round(frac * n_atoms))
        left -= counts[t]
    counts[composition[-1][0]] = left
    h_count = counts.pop("H", 0) if n_h is None else n_h
    inner = []
    for t, c in counts.items():
        inner += [t] * c
    inner = list(rng.permutation(inner))
    types = inner + ["H"] * h_count
    types = types[:n_atoms]
    xy = sites + rng.normal(0.0, jitter, size=sites.shape)
    z = rng.uniform(-zspread / 2, zspread / 2, size=n_atoms)
    q = rng.normal(0.0, qsigma, size=n_atoms)
    q -= q.mean()
    return types, np.column_stack([xy, z]), q


CLUSTER_PARAMS = {
    "C": (0.086, 3.4, 12.011, 0.0),
    "N": (0.17, 3.25, 14.007, 0.0),
    "H": (0.03, 2.42, 1.008, 0.0),
    # O is both a surface type and the tip type; its charge line is the tip's
    # charge (parse.cpp:626-631) because surface charges come from the xyz file.
    "O": (TIP[1], TIP[2], 15.999, -0.1),
    DUMMY[0]: (DUMMY[1], DUMMY[2], 0.0, 0.0),
}


def cluster_60(seed: int = 1234, area: float = 20.0, step: float = 0.05,
               zhigh: float = 10.0, zlow: float = 6.0, dz: float = 0.1,
               n_atoms: int = 60, **opt) -> ScanInput:
    """60-atom C/N/O/H cluster, Coulomb on, Morse (0.1, 1.5, 3.2) for tip-O."""
    rng = np.random.default_rng(seed)
    types, pos, q = planar_molecule(n_atoms, rng)
    o = base_options(area=f"{area} {area}", dx=step, dy=step, zhigh=zhigh, zlow=zlow,
                     dz=dz, coulomb="on")
    o.update({k: str(v) for k, v in opt.items()})
    return ScanInput("cluster_60", types, pos, q, dict(CLUSTER_PARAMS),
                     [("O", "O", "morse", 0.1, 1.5, 3.2)], (0.5, 0.0), o)


def naphthalene(cc: float = 1.40, ch: float = 1.09) -> tuple:
    """C10H8 in the xy plane: two fused hexagons (C-C cc) with H at ch."""
    carbons = []
    for cx in (-cc * math.sqrt(3) / 2, cc * math.sqrt(3) / 2):
        for k in range(6):
            ang = math.radians(30 + 60 * k)
            p = (cx + cc * math.cos(ang), cc * math.sin(ang))
            if all(math.hypot(p[0] - q[0], p[1] - q[1]) > 0.1 for q in carbons):
                carbons.append(p)
    hydrogens = []
    for p in carbons:
        if abs(p[0]) < 1e-6:
            continue                          # the two shared carbons carry no H
        d = np.array(p) - np.array((math.copysign(cc * math.sqrt(3) / 2, p[0]), 0.0))
        d /= np.linalg.norm(d)
        hydrogens.append(tuple(np.array(p) + ch * d))
    pos = [(x, y, 0.0) for x, y in carbons] + [(x, y, 0.0) for x, y in hydrogens]
    return ["C"] * len(carbons) + ["H"] * len(hydrogens), np.array(pos)


def flexible_naphthalene(seed: int = 21, area: float = 1.0, step: float = 0.5,
                         zhigh: float = 10.0, zlow: float = 8.0, dz: float = 0.2,
                         **opt) -> ScanInput:
    """Flexible C10H8 and a separate H2, with charges: free atoms, two
    XY-tethered hydrogens and one fixed carbon; bond / angle / dihedral /
    substrate parameters and topobonds for C-C, C-H and H-H (parse.cpp:699-782)."""
    rng = np.random.default_rng(seed)
    types, pos = naphthalene()
    # a separate H2 beside the ring: non-bonded pairs between the fragments
    types = types + ["H", "H"]
    pos = np.vstack([pos, [[4.6, -0.37, 0.3], [4.6, 0.37, 0.3]]])
    pos = pos + rng.normal(0.0, 0.01, pos.shape) * np.array([1.0, 1.0, 0.0])
    q = rng.normal(0.0, 0.1, len(types))
    q -= q.mean()
    fixed = np.zeros(len(types), dtype=int)
    fixed[len(types) - 3] = 2
    fixed[len(types) - 5] = 2
    fixed[0] = 1
    params = {"C": (0.086, 3.4, 12.011, 0.0), "H": (0.03, 2.5, 1.008, 0.0),
              TIP[0]: (TIP[1], TIP[2], 15.999, -0.1), DUMMY[0]: (DUMMY[1], DUMMY[2], 0.0, 0.0)}
    o = base_options(area=f"{area} {area}", dx=step, dy=step, zhigh=zhigh, zlow=zlow, dz=dz,
                     coulomb="on", flexible="on")
    o.update({k: str(v) for k, v in opt.items()})
    spec = ScanInput("naph", types, pos, q, params, [], (0.5, 0.0), o, None, fixed)
    spec.extra_param_lines = ["bond 50.0", "angle 20.0", "dihedral 2.0",
                              "substrate 0.1 3.0 3.0 7.5 1.0",
                              "topobond C C 1.40", "topobond C H 1.09", "topobond H H 0.74"]
    return spec


def write_cube(path: str, values: np.ndarray, voxel: np.ndarray, origin) -> None:
    """Gaussian cube in Angstrom units (negative voxel counts, cube_io.cpp:108-111)."""
    n0, n1, n2 = values.shape
    with open(path, "w") as f:
        f.write("synthetic Hartree potential\nsum of Gaussian charges on a compensating background\n")
        f.write(f"{0:5d} {origin[0]:12.6f} {origin[1]:12.6f} {origin[2]:12.6f}\n")
        for n, v in zip((n0, n1, n2), voxel):
            f.write(f"{-n:5d} {v[0]:12.6f} {v[1]:12.6f} {v[2]:12.6f}\n")
        flat = values.reshape(n0 * n1, n2)
        for row in flat:
            for s in range(0, n2, 6):
                f.write(" ".join(f"{x:13.5e}" for x in row[s:s + 6]) + "\n")


def gaussian_potential(pos: np.ndarray, q: np.ndarray, cell: np.ndarray, n: tuple,
                       width: float = 0.5) -> np.ndarray:
    """Periodic potential (Hartree/e) of Gaussian charges on a neutralising background.

    The charges are splatted onto the voxel grid as normalised Gaussians
    (periodic wrap, +-4 widths), then the Poisson equation is solved by FFT on
    the orthorhombic cell: V(k) = 4 pi rho(k) / k^2 with V(0) = 0 (the
    background), in e/A, converted e/A -> Hartree/e (1 e/A = BOHR Hartree).
    """
    n0, n1, n2 = n
    L = np.array([cell[0][0], cell[1][1], cell[2][2]])
    h = L / np.array(n)
    rho = np.zeros((n0, n1, n2))
    half = [int(math.ceil(4 * width / h[a])) for a in range(3)]
    offs = [np.arange(-half[a], half[a] + 1) for a in range(3)]
    for a in range(len(q)):
        idx, wts = [], []
        for d in range(3):
            c = pos[a, d] / h[d]
            i0 = int(math.floor(c))
            ii = i0 + offs[d]
            r = (ii - c) * h[d]
            idx.append(np.mod(ii, n[d]))
            wts.append(np.exp(-0.5 * (r / width) ** 2))
        block = q[a] * wts[0][:, None, None] * wts[1][None, :, None] * wts[2][None, None, :]
        rho[np.ix_(idx[0], idx[1], idx[2])] += block
    # normalise each Gaussian's discrete sum to its charge
    norm = (np.sqrt(2 * np.pi) * width) ** 3 / h.prod()
    rho /= norm * h.prod()
    k0 = 2 * np.pi * np.fft.fftfreq(n0, d=h[0])
    k1 = 2 * np.pi * np.fft.fftfreq(n1, d=h[1])
    k2 = 2 * np.pi * np.fft.rfftfreq(n2, d=h[2])
    K2 = k0[:, None, None] ** 2 + k1[None, :, None] ** 2 + k2[None, None, :] ** 2
    rho_k = np.fft.rfftn(rho)
    with np.errstate(divide="ignore", invalid="ignore"):
        v_k = np.where(K2 > 0, 4 * np.pi * rho_k / K2, 0.0)
    v = np.fft.irfftn(v_k, s=(n0, n1, n2), axes=(0, 1, 2))
    return v * BOHR


def slab(seed: int = 7, nlx: int = 16, nly: int = 32, layers: int = 4,
         cell=(40.0, 40.0, 30.0), cube_n=(160, 160, 120), pixels: int = 512,
         step: float = 0.2, zhigh: float = 16.0, zlow: float = 12.0, dz: float = 0.1,
         rigidgrid: bool = True, external: bool = True, tip_charge: float = -0.1,
         shear: float = 0.0, **opt) -> ScanInput:
    """Periodic slab (layers of nlx x nly sites), vdw_pbc, optional cube and grid.

    shear tilts the cell's b vector to (shear b, b, 0): the atoms keep their
    fractional coordinates and the cube its values, on sheared voxels (a
    non-orthogonal cube basis)."""
    rng = np.random.default_rng(seed)
    a, b, c = cell
    xs = (np.arange(nlx) + 0.5) * (a / nlx)
    ys = (np.arange(nly) + 0.5) * (b / nly)
    pos, types = [], []
    for L in range(layers):
        for i, x in enumerate(xs):
            for j, y in enumerate(ys):
                pos.append((x, y, 10.0 + 2.0 * L))
                types.append("C" if (i + j + L) % 2 == 0 else "N")
    frac_pos = np.array(pos)                 # orthorhombic frame (fractional x cell)
    pos = frac_pos.copy()
    pos[:, 0] += shear * pos[:, 1]           # (shear b, b, 0) for the b vector
    q = rng.normal(0.0, 0.3, size=len(pos))
    params = {"C": (0.086, 3.4, 12.011, 0.0), "N": (0.17, 3.25, 14.007, 0.0),
              TIP[0]: (TIP[1], TIP[2], 15.999, tip_charge), DUMMY[0]: (DUMMY[1], DUMMY[2], 0.0, 0.0)}
    area = step * (pixels - 1)
    o = base_options(area=f"{area!r} {area!r}", dx=step, dy=step, zhigh=zhigh, zlow=zlow,
                     dz=dz, vdw_pbc="on", rigidgrid="on" if rigidgrid else "off")
    if not external:
        o.update(cell_a=f"{a} 0 0", cell_b=f"{_fmt(shear * b)} {b} 0", cell_c=f"0 0 {c}")
    cube = None
    if external:
        o["use_external_potential"] = "on"
        voxel = np.diag([a / cube_n[0], b / cube_n[1], c / cube_n[2]])
        voxel[1, 0] = shear * b / cube_n[1]
        v = gaussian_potential(frac_pos, q, np.diag(cell), cube_n)
        cube = {"values": v, "voxel": voxel, "origin": (0.0, 0.0, 0.0)}
    o.update({k: str(v) for k, v in opt.items()})
    return ScanInput("slab", types, pos, None, params, [], (0.5, 0.0), o, cube)


def molecule_batch(n_scans: int = 256, seed: int = 99, grids=(64, 128, 256),
                   atoms=(20, 400), step: float = 0.1, zhigh: float = 10.0,
                   zlow: float = 6.0, dz: float = 0.1, **opt) -> list:
    """Independent rigid scans of seeded planar molecules, LJ + Coulomb."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = math.log(atoms[0]), math.log(atoms[1])
    for s in range(n_scans):
        n = int(round(math.exp(rng.uniform(lo, hi))))
        g = int(rng.choice(grids))
        types, pos, q = planar_molecule(n, rng)
        area = step * (g - 1)
        o = base_options(area=f"{area!r} {area!r}", dx=step, dy=step, zhigh=zhigh,
                         zlow=zlow, dz=dz, coulomb="on")
        o.update({k: str(v) for k, v in opt.items()})
        params = dict(CLUSTER_PARAMS)
        out.append(ScanInput(f"mol{s:03d}", types, pos, q, params, [], (0.5, 0.0), o))
    return out
