"""Synthetic workloads of the Steinbach step, and writers for input files in
the reference's formats.

Physical parameters are those of the reference's sample input
(zhubq/PhaseField, C++-openmp-cuda/build/log_file.txt:33-62 for mobilities,
interface energies and carbon diffusivities; build/thermo_data.txt:4-29 for the
entropy and PARA phase-diagram lines; cutoff 1e-5 from log_file.txt:12).  Mn is
an extension with no reference counterpart: D_Mn = 1e-6 * D_C per phase with the
carbon activation energies, and a linear partition c_Mn,p proportional to
(1, 2, 10) for ferrite, austenite, cementite.

The microstructures are seeded and synthetic (periodic Voronoi ferrite grains,
austenite nuclei, cementite particles, tanh interfaces); no dataset is involved.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

from . import CONFIG_DIR, PF_PREC_FP32C, PF_PREC_FP64, PfInitSpec

# (m0 [um^4/J/s], Q [J/mol]) for pairs (1,1),(1,2),(1,3),(2,2),(2,3),(3,3)
MOBILITY = [(24e29, 360000.0), (200.0e16, 140000.0), (0.0e26, 332826.0),
            (0.0e28, 360000.0), (0.0e28, 360000.0), (0.0e-33, 16000000.0)]
# interface energy [J/um^2], same pair order
SIGMA = [0.76e-12, 0.4e-12, 0.7e-12, 0.76e-12, 0.94e-12, 0.3e-12]
# carbon diffusivity (D0 [um^2/s], Q [J/mol]) in ferrite, austenite, cementite
D_CARBON = [(0.1e8, 122500.0), (0.15e8, 142000.0), (0.0e8, 142000.0)]
D_MN = [(10.0, 122500.0), (15.0, 142000.0), (0.0, 142000.0)]
MN_RATIO = (1.0, 2.0, 10.0)

THERMO_TEXT = """\
# three phases: 1 ferrite, 2 austenite, 3 cementite
# mixed-mode driving force: dG = k*(c - c_eq)/(dc/dT), entropy k_ij = a*T + b [J/K/um^3]
# entropy lines: i j a b
1 2 0. 0.2e-12
1 3 0. 0.25e-12
2 3 0. 1.0e-12
# equilibrium lines (wt% = a*T^2 + b*T + c), three blocks: NPLE1, NPLE2, PARA
# each block lists the six ordered pairs: i j a b c
# NPLE1
1 2 1e-4 1e-2 0.1
2 1 1e-2 1e-2 0.02
1 3 0 1e-2 0.001
3 1 0 1e-3 0.01
2 3 0 -1e-3 0.1
3 2 0 -9e-3 0.1
# NPLE2
1 2 1e-4 1e-2 0.1
2 1 1e-2 1e-2 0.02
1 3 0 1e-2 0.001
3 1 0 1e-3 0.01
2 3 0 -1e-3 0.1
3 2 0 -9e-3 0.1
# PARA
1 2 0. -1e-4 0.11
2 1 0. -5e-3 5.395
1 3 0 1e-2 0.001
3 1 0 1e-3 0.01
2 3 0 -1e-3 0.1
3 2 0 -9e-3 0.1
"""

_PAIRS = ["ferrite-ferrite", "ferrite-austenite", "ferrite-cementite",
          "austenite-austenite", "austenite-cementite", "cementite-cementite"]
_PHASES = ["ferrite", "austenite", "cementite"]


# Selects the Fortran intercritical-annealing model's thermodynamics
# (Fortran_openmp_phase_field/PFM/src/sparse.f90:797-923): piecewise polynomial
# para lines and the linear austenite driving force, all coefficients built in.
THERMO_F90_TEXT = """F90_POLYNOMIAL
# para/NPLE lines of the Fortran model (sparse.f90:797-923); no coefficients here
"""


# Solute-drag parameters of the Fortran model's sample input
# (Fortran_openmp_phase_field/PFM/example/log_file.txt, last block): binding
# energy 10000 J/mol, v_m0 1e11 um/s, Q_sd 247650 J/mol.
F90_DRAG_LINE = "SOLUTE_DRAG 10000. 1.0e11 247650.\n"


def write_thermo(path: str, model: str = "linear", coherent_npp0: int | None = None) -> str:
    """model: "linear" (the reference's sample lines), "f90" (the Fortran
    model's thermodynamics), "f90avg" (that, plus the interface-averaged
    carbon of sparse.f90:184-255) or "f90drag" (that, plus the solute drag of
    sparse.f90:326-360 with the Fortran sample's parameters).  coherent_npp0
    (an "f90" model): add the coherent-grain mobility of sparse.f90:298-315,
    ferrite ids up to coherent_npp0 forming the initial class."""
    text = {"linear": THERMO_TEXT, "f90": THERMO_F90_TEXT,
            "f90avg": THERMO_F90_TEXT + "AVERAGED_INTERFACE_CARBON\n",
            "f90drag": THERMO_F90_TEXT + F90_DRAG_LINE}[model]
    if coherent_npp0 is not None:
        if model == "linear":
            raise ValueError("the coherent-grain mobility is an option of the Fortran model's thermodynamics")
        text += f"COHERENT_MOBILITY {int(coherent_npp0)}\n"
    with open(path, "w") as f:
        f.write(text)
    return path


def write_config(path: str, *, grid, dx=0.5, i_intf=6, cutoff=1e-5, T=1023.0, end_time=1.0e6,
                 directory="pf_output", thermo_file="thermo_steel.txt", mn=True, num_nuclei=0,
                 num_grain=(20, 0, 0), init_conc=(0.1, 0.1, 0.1), timestep_output=1.0e30,
                 micro_out=0, T_path=None, mobility=None, sigma=None, d_carbon=None, d_mn=None,
                 mn_ratio=MN_RATIO) -> str:
    """Write a configuration file in the reference's positional format
    (phase_field.cpp:166-330): a prompt line before every value."""
    ix, iy, iz = grid
    mob = mobility or MOBILITY
    sig = sigma or SIGMA
    dc = d_carbon or D_CARBON
    dm = d_mn or D_MN
    path_T = T_path or [(0.0, T), (end_time, T)]
    L = ["output folder?", directory,
         "grid size (2D: iz=1; 1D: iy=iz=1)", "number of cells along x, y, z", "[ix iy iz]?",
         f"{ix} {iy} {iz}",
         "cell size (um)?", f"{dx!r}",
         "interface width (cells)?", f"{i_intf}",
         "phase-field cutoff?", f"{cutoff!r}",
         "grain numbers (ferrite austenite cementite)?", " ".join(str(g) for g in num_grain),
         "initial phase fractions?", "0.5 0.5 0.",
         "initial phase concentrations (wt%)?", " ".join(repr(float(c)) for c in init_conc),
         "temperature path: number of points, then (time [s], T [K]) pairs?", f"{len(path_T)}"]
    L += [f"{t!r} {TT!r}" for t, TT in path_T]
    L += ["rolling reduction?", "0.",
          "initial smoothing iterations?", "0",
          "output interval (s)?", f"{timestep_output!r}",
          "write VTI microstructure files (1/0)?", f"{int(micro_out)}",
          "number of nuclei?", f"{num_nuclei}"]
    for name, (m0, q) in zip(_PAIRS, mob):
        L += [f"{name} mobility: m0 [um^4/J/s], Q [J/mol]?", f"{m0!r} {q!r}"]
    for name, s in zip(_PAIRS, sig):
        L += [f"{name} interface energy [J/um^2]?", f"{s!r}"]
    for name, (d0, q) in zip(_PHASES, dc):
        L += [f"carbon diffusivity in {name}: D0 [um^2/s], Q [J/mol]?", f"{d0!r} {q!r}"]
    L += ["thermodynamic file?", thermo_file, "use the GPU (1/0)?", "1"]
    if mn:
        for name, (d0, q) in zip(_PHASES, dm):
            L += [f"Mn diffusivity in {name}: D0 [um^2/s], Q [J/mol]?", f"{d0!r} {q!r}"]
        L += ["Mn partition ratios (ferrite austenite cementite)?", " ".join(repr(float(r)) for r in mn_ratio)]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")
    return path


@dataclass
class Workload:
    """One configuration of the step: grid, temperature, microstructure, steps."""

    name: str
    grid: tuple
    T: float
    steps: int
    precision: int
    n_grains: int
    n_nuclei: int
    nucleus_radius: float
    n_particles: int = 0
    particle_radius: float = 2.0
    C0: tuple = (0.10, 1.5)
    C_noise: tuple = (0.0, 0.0)
    width: float = 6.0
    dx: float = 0.5
    seed: int = 0
    max_slots: int = 4
    extra: dict = field(default_factory=dict)

    @property
    def N(self) -> int:
        return self.grid[0] * self.grid[1] * self.grid[2]

    def spec(self) -> PfInitSpec:
        s = PfInitSpec()
        s.seed = self.seed
        s.n_grains = self.n_grains
        s.n_nuclei = self.n_nuclei
        s.nucleus_radius = self.nucleus_radius
        s.n_particles = self.n_particles
        s.particle_radius = self.particle_radius
        s.width = self.width
        s.C0[0], s.C0[1] = self.C0
        s.C_noise[0], s.C_noise[1] = self.C_noise
        s.max_slots = self.max_slots
        return s

    def write_inputs(self, directory: str, grid=None) -> str:
        """Write config + thermo files for this workload (optionally on another grid)."""
        os.makedirs(directory, exist_ok=True)
        write_thermo(os.path.join(directory, "thermo_steel.txt"))
        return write_config(os.path.join(directory, f"{self.name}.txt"), grid=grid or self.grid, dx=self.dx,
                            T=self.T, num_grain=(self.n_grains, 0, 0), num_nuclei=self.n_nuclei,
                            directory=os.path.join(directory, "out_" + self.name))


def _particles(area_fraction: float, grid, r: float) -> int:
    return int(round(area_fraction * grid[0] * grid[1] / (math.pi * r * r)))


WORKLOADS = {
    # 2D plain FP64, CPU-runnable: 256^2, 20 ferrite grains, 30 nuclei r=3.
    "2d256": Workload("2d256", (256, 256, 1), 1023.0, 1000, PF_PREC_FP64, 20, 30, 3.0),
    # 3D FP32 compensated vs FP64: 256^3, 200 grains, 2000 nuclei r=2, noise 0.02 wt%.
    "3d256": Workload("3d256", (256, 256, 256), 1013.0, 2000, PF_PREC_FP32C, 200, 2000, 2.0,
                      C_noise=(0.02, 0.02)),
    # 2D three phases (cementite r=2 at 0.5% area), 512^2.
    "2d512cem": Workload("2d512cem", (512, 512, 1), 1023.0, 2000, PF_PREC_FP32C, 20, 30, 3.0,
                         n_particles=_particles(0.005, (512, 512), 2.0), particle_radius=2.0),
    # Large 3D: 512^3, 1000 grains, 20000 nuclei.
    "3d512": Workload("3d512", (512, 512, 512), 1023.0, 10000, PF_PREC_FP32C, 1000, 20000, 2.0),
}


def packaged_config(name: str) -> str:
    return os.path.join(CONFIG_DIR, f"{name}.txt")


@dataclass
class EnsembleDomain:
    grid: tuple
    T: float
    C0: float
    n_grains: int
    n_nuclei: int
    seed: int


def ensemble(n_domains: int = 64, seed: int = 0, sizes=(128, 512), T_range=(993.0, 1053.0),
             C_range=(0.05, 0.20)) -> list:
    """The batched ensemble: square 2D domains with sides drawn uniform from the
    multiples of 32 in [sizes], temperature and carbon drawn uniform from the
    ranges, and per-domain grain and nucleus densities, all from one seed."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sides = np.arange(sizes[0], sizes[1] + 1, 32)
    out = []
    for d in range(n_domains):
        L = int(rng.choice(sides))
        T = float(rng.uniform(*T_range))
        C0 = float(rng.uniform(*C_range))
        grains = max(2, int(round(L * L / float(rng.uniform(2000.0, 6000.0)))))
        nuclei = int(round(L * L * float(rng.uniform(2e-4, 8e-4))))
        out.append(EnsembleDomain((L, L, 1), T, C0, grains, nuclei, int(seed * 1000 + d)))
    return out


def ensemble_inputs(directory: str, domains: list) -> list:
    """Write one config file per ensemble domain; returns their paths."""
    os.makedirs(directory, exist_ok=True)
    write_thermo(os.path.join(directory, "thermo_steel.txt"))
    paths = []
    for d, dom in enumerate(domains):
        paths.append(write_config(os.path.join(directory, f"ens{d:03d}.txt"), grid=dom.grid, T=dom.T,
                                  num_grain=(dom.n_grains, 0, 0), num_nuclei=dom.n_nuclei,
                                  directory=os.path.join(directory, f"out{d:03d}")))
    return paths


def ensemble_spec(dom: EnsembleDomain) -> PfInitSpec:
    s = PfInitSpec()
    s.seed = dom.seed
    s.n_grains = dom.n_grains
    s.n_nuclei = dom.n_nuclei
    s.nucleus_radius = 3.0
    s.width = 6.0
    s.C0[0], s.C0[1] = dom.C0, 1.5
    s.max_slots = 4
    return s
