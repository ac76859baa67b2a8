"""Problem set-up and the host-side mirror of the reference's driver.

``Problem`` owns everything the reference's main() assembles before its
time loop (src/main.cpp:32-300): the preprocessed macro and micro meshes,
the effective-conductivity table, the two soils, ``user_data`` and the
initial state.  ``Context`` is the GPU hot path behind the C-ABI, and
``run_to_end`` is the reference's ``while (t < tend) exprem(...)`` loop
(src/main.cpp:313-341).

Configurations (seeded, synthetic; the reference publishes no dataset):
  * ``config1``  -- 21x21-node triangulated macro mesh, 11x11-node square
    inclusion per cell, Dirichlet top, N = 97,241.
  * ``config2``  -- 201x201 macro nodes, 21x21 micro per cell with per-cell
    inclusion size U(0.3, 0.7), Dirichlet strip x in [0.25, 0.75],
    h0 = -5 + N(0, 0.1^2); N = 35,320,401.
  * ``fixture10`` -- the shape of the reference's own test (10x10
    quadrilateral macro mesh, irregular triangulated inclusion, tabulated
    full Keff tensor, flux / free-drainage / no-flow BCs, model_type 3).
"""
import ctypes as C

import numpy as np

from . import capi, meshgen
from .capi import check, ptr

GENERATOR_SEED = 20261203
EVAL_SEED = 7

# van Genuchten materials of the configurations (m and day units)
SOIL_A = dict(Ksat=0.054, thetar=0.03, thetas=0.37, alpha=2.8, n=2.24)
SOIL_B = dict(Ksat=0.001, thetar=0.10, thetas=0.45, alpha=0.5, n=1.40)


def make_soil(Ksat, thetar, thetas, alpha, n):
    s = capi.Soil()
    s.Ksat, s.thetar, s.thetas, s.alpha, s.n = Ksat, thetar, thetas, alpha, n
    s.m = 1.0 - 1.0 / n                      # as src/main.cpp:127,140
    return s


def default_options(lib=None, **kw):
    """The reference's solver defaults (src/set_exprem_options.cpp:16-26)
    with overrides.  lib: the library that provides tsr_set_exprem_options
    (default: this package's)."""
    lib = lib or capi.load()
    o = capi.ExpremOptions()
    check(lib.tsr_set_exprem_options(C.byref(o)), "tsr_set_exprem_options")
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Problem:
    """Preprocessed two-scale problem (host memory)."""

    def __init__(self, macro, micro, keff_rows, epsA, soilA, soilB, *, macro_bc,
                 model_type=3, boundary_flux=0.0, dirichlet_h=0.0, specific_storage=1e-6,
                 kface=0, cell_scale=None, logh_first=None, logr=None, name="",
                 templates=None, cell_template=None, cell_soilB=None, scenarios=1,
                 scen_soilA=None, scen_keff_scale=None, lib=None):
        """micro: the micro mesh of every cell; or, for the batched form,
        templates (list of micro meshes) with cell_template[k] naming the
        template of cell k and optional per-cell material B (list of dicts).
        lib: the library whose mesh preprocessing builds the geometry
        (tsr_macro_mesh_build / tsr_micro_mesh_build and their frees;
        default: this package's)."""
        lib = lib or capi.load()
        self._lib = lib
        self.name = name
        self._bc = np.ascontiguousarray(macro_bc, dtype=np.int32)
        if isinstance(macro, capi.MacroMesh):
            self.macro = macro             # preprocessed by this library's reader (owned here)
        else:
            self.macro = capi.MacroMesh()
            check(lib.tsr_macro_mesh_build(macro.nv, macro.n_nodes, ptr(macro.xy), macro.n_elems,
                                           ptr(macro.elems), macro.bedges.size // 3, ptr(macro.bedges),
                                           ptr(self._bc), C.byref(self.macro)), "tsr_macro_mesh_build")
        if templates is not None:
            micro = templates[0]
        self._tpl = None
        if templates is not None:
            self._tpl = (capi.MicroMesh * len(templates))()
            for i, t in enumerate(templates):
                check(lib.tsr_micro_mesh_build(t.cell[0], t.cell[1], t.nv, t.n_nodes, ptr(t.xy),
                                               t.n_elems, ptr(t.elems), t.bedges.size // 3,
                                               ptr(t.bedges), C.byref(self._tpl[i])),
                      "tsr_micro_mesh_build")
        if isinstance(micro, capi.MicroMesh):
            self.micro = micro
        else:
            self.micro = capi.MicroMesh()
            check(lib.tsr_micro_mesh_build(micro.cell[0], micro.cell[1], micro.nv, micro.n_nodes,
                                           ptr(micro.xy), micro.n_elems, ptr(micro.elems),
                                           micro.bedges.size // 3, ptr(micro.bedges),
                                           C.byref(self.micro)), "tsr_micro_mesh_build")
        self._keff_owned = isinstance(keff_rows, capi.Keff)
        if self._keff_owned:
            self.keff = keff_rows          # read by this library's reader (owned here)
        else:
            rows = np.asarray(keff_rows, dtype=np.float64)   # (n, 5): log10|h|, K11, K12, K21, K22
            self._logh = np.ascontiguousarray(rows[:, 0])
            self._kv = np.ascontiguousarray(rows[:, 1:].T.ravel())   # component-major
            self.keff = capi.Keff()
            self.keff.epsilonA = epsA
            self.keff.no_hvalues = len(rows)
            self.keff.logh_first = rows[0, 0] if logh_first is None else logh_first
            self.keff.logr = (rows[1, 0] - rows[0, 0]) if logr is None else logr
            self.keff.logh_values = ptr(self._logh)
            self.keff.Keff_values = ptr(self._kv)
        self.soilA = make_soil(**soilA) if isinstance(soilA, dict) else soilA
        self.soilB = make_soil(**soilB) if isinstance(soilB, dict) else soilB
        self.soilB_dict = dict(soilB) if isinstance(soilB, dict) else None
        self.ud = capi.UserData()
        self.ud.macro_mesh = self.macro
        self.ud.micro_mesh = self.micro
        self.ud.effective_conductivity = self.keff
        self.ud.soilA = self.soilA
        self.ud.soilB = self.soilB
        self.ud.boundary_flux = boundary_flux
        self.ud.model_type = model_type
        self.ud.NUM_THREADS = 1
        self.Mn = self.macro.no_nodes
        self.Ne = self.macro.no_elements
        self.mn = self.micro.no_nodes
        self._scale = None if cell_scale is None else np.ascontiguousarray(cell_scale, np.float64)
        self.ext = capi.ModelExt()
        self.ext.dirichlet_h = dirichlet_h
        self.ext.specific_storage = specific_storage
        self.ext.kface_mode = kface
        self.ext.cell_scale = ptr(self._scale)
        if templates is not None:
            self.cell_template = np.ascontiguousarray(cell_template, dtype=np.int32)
            mns = np.array([t.no_nodes for t in self._tpl], dtype=np.int64)
            self.cell_nodes = mns[self.cell_template]
            self.cell_off = self.Mn + np.concatenate([[0], np.cumsum(self.cell_nodes)[:-1]])
            self.N = int(self.Mn + self.cell_nodes.sum())
            self.ext.n_templates = len(templates)
            self.ext.templates = C.cast(self._tpl, C.POINTER(capi.MicroMesh))
            self.ext.cell_template = ptr(self.cell_template)
            if cell_soilB is not None:
                self._soils = (capi.Soil * self.Ne)(*[make_soil(**s) for s in cell_soilB])
                self.ext.cell_soilB = C.cast(self._soils, C.POINTER(capi.Soil))
        else:
            self.cell_template = None
            self.cell_nodes = np.full(self.Ne, self.mn, dtype=np.int64)
            self.cell_off = self.Mn + self.mn * np.arange(self.Ne, dtype=np.int64)
            self.N = self.Mn + self.Ne * self.mn
        if templates is None and cell_soilB is not None:
            self._soils = (capi.Soil * self.Ne)(*[make_soil(**s) for s in cell_soilB])
            self.ext.cell_soilB = C.cast(self._soils, C.POINTER(capi.Soil))
        # scenario-major layout of the unknowns: [macro_s | cells_s] per scenario
        self.S = scenarios
        Mn_s, Ne_s = self.Mn // scenarios, self.Ne // scenarios
        self.node_off = np.empty(self.Mn, dtype=np.int64)
        self.scen_start = np.zeros(scenarios + 1, dtype=np.int64)
        off = 0
        cell_off = np.empty(self.Ne, dtype=np.int64)
        for s in range(scenarios):
            self.scen_start[s] = off
            self.node_off[s * Mn_s:(s + 1) * Mn_s] = off + np.arange(Mn_s)
            off += Mn_s
            cn = self.cell_nodes[s * Ne_s:(s + 1) * Ne_s]
            cell_off[s * Ne_s:(s + 1) * Ne_s] = off + np.concatenate([[0], np.cumsum(cn)[:-1]])
            off += int(cn.sum())
        self.scen_start[scenarios] = off
        self.cell_off = cell_off
        if scenarios > 1:
            self.ext.scenarios = scenarios
            if scen_soilA is not None:
                self._scenA = (capi.Soil * scenarios)(*[make_soil(**s) for s in scen_soilA])
                self.ext.scen_soilA = C.cast(self._scenA, C.POINTER(capi.Soil))
            if scen_keff_scale is not None:
                self._kscale = np.ascontiguousarray(scen_keff_scale, dtype=np.float64)
                self.ext.scen_keff_scale = ptr(self._kscale)
        self.ud.N = self.N
        self.dirichlet_h = dirichlet_h
        nv, Ne = self.macro.no_verts, self.Ne
        bce = capi.as_array(self.macro.boundary_condition_edges, nv * Ne, np.int32)
        el = capi.as_array(self.macro.elements, nv * Ne, np.int32)
        mask = np.zeros(self.Mn, bool)
        for j in range(nv):
            d = bce[j * Ne:(j + 1) * Ne] == 5
            mask[el[j * Ne:(j + 1) * Ne][d]] = True
            mask[el[((j + 1) % nv) * Ne:((j + 1) % nv + 1) * Ne][d]] = True
        self.dirichlet_nodes = mask
        self.options = default_options(lib)
        self.tspan = np.array([0.0])
        self.tend = 1.0

    def set_learned(self, learned, kappa=None):
        """Learned-closure layout (one scenario): cell k with learned[k]
        carries one unknown instead of its micro nodes; kappa (2 Ne) are the
        closure coefficients (kQ, kT) per cell.  Contexts built afterwards
        can switch cells at run time (tsr_closure_set_learned)."""
        assert self.S == 1
        if not hasattr(self, "cell_nodes_full"):
            self.cell_nodes_full = self.cell_nodes.copy()
            self.N_full = self.N
        self._learned = np.ascontiguousarray(learned, dtype=np.int32)
        self._kappa = (np.zeros(2 * self.Ne) if kappa is None
                       else np.ascontiguousarray(kappa, dtype=np.float64))
        self.ext.cell_learned = ptr(self._learned)
        self.ext.closure_coef = ptr(self._kappa)
        self.cell_nodes = np.where(self._learned != 0, 1, self.cell_nodes_full).astype(np.int64)
        self.cell_off = self.Mn + np.concatenate([[0], np.cumsum(self.cell_nodes)[:-1]]).astype(np.int64)
        self.N = int(self.Mn + self.cell_nodes.sum())
        self.scen_start = np.array([0, self.N], dtype=np.int64)
        self.ud.N = self.N

    def initial_state(self, h0=-5.0, noise=0.0, seed=EVAL_SEED):
        """h0 (a number, or one number per scenario) plus optional noise;
        Dirichlet nodes at their head."""
        h0 = np.broadcast_to(np.asarray(h0, dtype=np.float64), (self.S,))
        u = np.empty(self.N, dtype=np.float64)
        for s in range(self.S):
            u[self.scen_start[s]:self.scen_start[s + 1]] = h0[s]
        if noise > 0.0:
            u += np.random.default_rng(seed).normal(0.0, noise, self.N)
        u[self.node_off[self.dirichlet_nodes]] = self.dirichlet_h
        return u

    def scenario(self, u, s):
        """The unknowns of scenario s (a view)."""
        return u[self.scen_start[s]:self.scen_start[s + 1]]

    def array(self, name, n, dtype=np.float64, micro=False):
        s = self.micro if micro else self.macro
        return capi.as_array(getattr(s, name), n, dtype)

    def close(self):
        lib = self._lib
        if self.macro.elements:
            lib.tsr_macro_mesh_free(C.byref(self.macro))
        if self.micro.elements:
            lib.tsr_micro_mesh_free(C.byref(self.micro))
        if self._tpl is not None:
            for t in self._tpl:
                if t.elements:
                    lib.tsr_micro_mesh_free(C.byref(t))
            self._tpl = None
        if getattr(self, "_keff_owned", False) and self.keff.Keff_values:
            lib.tsr_keff_free(C.byref(self.keff))
            self._keff_owned = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def constant_keff_rows(k=0.02):
    """A two-row table (log10|h| = 2 and -2) holding an isotropic constant."""
    return [[2.0, k, 0.0, 0.0, k], [-2.0, k, 0.0, 0.0, k]]


def config1(kface=0, lib=None):
    """21x21 macro nodes (800 triangles), 11x11-node square inclusion of side
    0.5 per cell, cell = macro spacing 0.05 m; Dirichlet h = -0.1 on the top
    side, no flow elsewhere; h0 = -5; EXPREM tol 1e-6, Krylov <= 30,
    t_end = 1 day, 10 saved times."""
    macro = meshgen.macro_unit_square(21)
    micro = meshgen.micro_square_inclusion(11, cell=0.05, side=0.5)
    p = Problem(macro, micro, constant_keff_rows(0.02), 0.75, SOIL_A, SOIL_B,
                macro_bc=[5, 2, 2, 2, 2], model_type=3, dirichlet_h=-0.1, kface=kface,
                name="config1", lib=lib)
    p.options = default_options(lib, AbsTol=1e-6, RelTol=1e-6, MaxKrylov=30)
    p.tend = 1.0
    p.tspan = np.concatenate([[10.0], np.linspace(0.1, 1.0, 10)])
    p.u0 = p.initial_state(-5.0)
    return p


def config2(n_macro=201, n_micro=21, seed=GENERATOR_SEED, eval_seed=EVAL_SEED, lib=None):
    """GPU-scale plain method: n_macro^2 macro nodes, n_micro^2 micro nodes
    per cell, inclusion side per cell U(0.3, 0.7) of the cell (a per-cell
    scale of the side-0.5 template), Dirichlet h = -0.1 on the top strip
    x in [0.25, 0.75], no flow elsewhere, h0 = -5 + N(0, 0.1^2) per unknown;
    EXPREM tol 1e-6, Krylov <= 40, t_end = 2 days."""
    h = 1.0 / (n_macro - 1)
    macro = meshgen.macro_unit_square(n_macro, segment=(0.25, 0.75))
    micro = meshgen.micro_square_inclusion(n_micro, cell=h, side=0.5)
    Ne = 2 * (n_macro - 1) ** 2
    side = np.random.default_rng(seed).uniform(0.3, 0.7, Ne)
    scale = side / 0.5
    epsA = 1.0 - (0.7 ** 3 - 0.3 ** 3) / (3 * 0.4)           # 1 - E[side^2]
    p = Problem(macro, micro, constant_keff_rows(0.02), epsA, SOIL_A, SOIL_B,
                macro_bc=[5, 2, 2, 2, 2], model_type=3, dirichlet_h=-0.1, cell_scale=scale,
                name="config2_%d_%d" % (n_macro, n_micro), lib=lib)
    p.options = default_options(lib, AbsTol=1e-6, RelTol=1e-6, MaxKrylov=40)
    p.tend = 2.0
    p.tspan = np.concatenate([[10.0], np.linspace(0.2, 2.0, 10)])
    p.u0 = p.initial_state(-5.0, noise=0.1, seed=eval_seed)
    return p


MICRO_SIDES = (5, 9, 15, 21, 31, 41)
MICRO_SIDE_P = (0.30, 0.25, 0.20, 0.12, 0.08, 0.05)


def config3(n_macro=151, seed=GENERATOR_SEED, eval_seed=EVAL_SEED, lib=None):
    """Batched form with uneven micro meshes: n_macro^2 macro nodes; per cell
    a micro mesh side from {5,9,15,21,31,41} (p = .30,.25,.20,.12,.08,.05), a
    square or disk inclusion (p = 0.5) of size U(0.2, 0.8) of the cell, and
    material B perturbed by lognormal factors (sigma 0.2 on alpha and Ks,
    0.05 on n).  Dirichlet top strip, EXPREM as config1."""
    h = 1.0 / (n_macro - 1)
    macro = meshgen.macro_unit_square(n_macro, segment=(0.25, 0.75))
    templates = []
    for n in MICRO_SIDES:
        templates.append(meshgen.micro_square_inclusion(n, cell=h, side=0.5))
        templates.append(meshgen.micro_disk_inclusion(n, cell=h, diameter=0.5))
    Ne = 2 * (n_macro - 1) ** 2
    rng = np.random.default_rng(seed)
    side = rng.choice(len(MICRO_SIDES), size=Ne, p=MICRO_SIDE_P)
    disk = rng.random(Ne) < 0.5
    size = rng.uniform(0.2, 0.8, Ne)
    tpl = (2 * side + disk).astype(np.int32)
    scale = size / 0.5
    fa = rng.lognormal(0.0, 0.2, Ne)
    fk = rng.lognormal(0.0, 0.2, Ne)
    fn = rng.lognormal(0.0, 0.05, Ne)
    soils = [dict(SOIL_B, alpha=SOIL_B["alpha"] * a, Ksat=SOIL_B["Ksat"] * k,
                  n=max(1.05, SOIL_B["n"] * n_)) for a, k, n_ in zip(fa, fk, fn)]
    frac = np.where(disk, np.pi * size ** 2 / 4.0, size ** 2)
    p = Problem(macro, None, constant_keff_rows(0.02), 1.0 - frac.mean(), SOIL_A, SOIL_B,
                macro_bc=[5, 2, 2, 2, 2], model_type=3, dirichlet_h=-0.1, cell_scale=scale,
                templates=templates, cell_template=tpl, cell_soilB=soils,
                name="config3_%d" % n_macro, lib=lib)
    p.options = default_options(lib, AbsTol=1e-6, RelTol=1e-6, MaxKrylov=30)
    p.tend = 1.0
    p.tspan = np.concatenate([[10.0], np.linspace(0.1, 1.0, 10)])
    p.u0 = p.initial_state(-5.0, noise=0.1, seed=eval_seed)
    return p


def union_mesh(mesh, copies):
    """`copies` disjoint copies of a macro mesh, block s numbered after s-1."""
    n, nv = mesh.n_nodes, mesh.nv
    xy = np.concatenate([np.tile(mesh.xy[:n], copies), np.tile(mesh.xy[n:], copies)])
    el = np.concatenate([mesh.elems + s * n for s in range(copies)])
    b = mesh.bedges.reshape(-1, 3)
    bed = np.concatenate([np.column_stack([b[:, 0] + s * n, b[:, 1] + s * n, b[:, 2]])
                          for s in range(copies)])
    return meshgen.Mesh(nv, xy, el, bed.ravel())


def config4(scenarios=64, n_macro=51, n_micro=15, seed=GENERATOR_SEED, eval_seed=EVAL_SEED,
            lib=None):
    """Ensemble: `scenarios` independent problems solved together, each on an
    n_macro^2 macro grid with n_micro^2 micro meshes (square inclusion of
    side 0.5), Dirichlet top h = -0.1, no flow elsewhere.  Per scenario:
    Ks_A ~ LogNormal(ln 0.054, 0.5), Ks_B ~ LogNormal(ln 0.001, 0.5),
    alpha_A ~ U(1.5, 4.0), n_A ~ U(1.8, 2.6), Keff scaled by Ks_A / 0.054,
    initial head U(-10, -1) m.  EXPREM tol 1e-6, Krylov <= 30, t_end = 1 d,
    each scenario with its own step size and Krylov dimension."""
    h = 1.0 / (n_macro - 1)
    base = meshgen.macro_unit_square(n_macro)
    macro = union_mesh(base, scenarios)
    micro = meshgen.micro_square_inclusion(n_micro, cell=h, side=0.5)
    rng = np.random.default_rng(seed)
    ksA = rng.lognormal(np.log(0.054), 0.5, scenarios)
    ksB = rng.lognormal(np.log(0.001), 0.5, scenarios)
    alA = rng.uniform(1.5, 4.0, scenarios)
    nA = rng.uniform(1.8, 2.6, scenarios)
    h0 = np.random.default_rng(eval_seed).uniform(-10.0, -1.0, scenarios)
    soilsA = [dict(SOIL_A, Ksat=k, alpha=a, n=n) for k, a, n in zip(ksA, alA, nA)]
    soilsB = [dict(SOIL_B, Ksat=k) for k in ksB]
    Ne_s = 2 * (n_macro - 1) ** 2
    cellB = [soilsB[s] for s in range(scenarios) for _ in range(Ne_s)]
    p = Problem(macro, micro, constant_keff_rows(0.02), 0.75, SOIL_A, SOIL_B,
                macro_bc=[5, 2, 2, 2, 2], model_type=3, dirichlet_h=-0.1, cell_soilB=cellB,
                scenarios=scenarios, scen_soilA=soilsA, scen_keff_scale=ksA / 0.054,
                name="config4_%dx%d_%d" % (scenarios, n_macro, n_micro), lib=lib)
    p.options = default_options(lib, AbsTol=1e-6, RelTol=1e-6, MaxKrylov=30)
    p.tend = 1.0
    p.tspan = np.array([0.0])
    p.h0 = h0
    p.u0 = p.initial_state(h0)
    p.scenario_params = dict(Ks_A=ksA, Ks_B=ksB, alpha_A=alA, n_A=nA, h0=h0)
    return p


def scenario_problem(ens, s, lib=None):
    """Scenario s of an ensemble as a standalone problem (same unknowns)."""
    pr = ens.scenario_params
    n_macro = int(round(np.sqrt(ens.Mn // ens.S)))
    h = 1.0 / (n_macro - 1)
    n_micro = int(round(np.sqrt(ens.mn)))
    macro = meshgen.macro_unit_square(n_macro)
    micro = meshgen.micro_square_inclusion(n_micro, cell=h, side=0.5)
    K = constant_keff_rows(0.02 * (pr["Ks_A"][s] / 0.054))    # the ensemble's scale, same rounding
    p = Problem(macro, micro, K, 0.75, dict(SOIL_A, Ksat=pr["Ks_A"][s], alpha=pr["alpha_A"][s],
                                            n=pr["n_A"][s]),
                dict(SOIL_B, Ksat=pr["Ks_B"][s]), macro_bc=[5, 2, 2, 2, 2], model_type=3,
                dirichlet_h=-0.1, name="scenario%d" % s, lib=lib)
    p.options = ens.options
    p.tend = ens.tend
    p.tspan = np.array([0.0])
    p.u0 = np.ascontiguousarray(ens.scenario(ens.u0, s))
    return p


def fixture10(boundary_flux=0.05, jitter=0.25, seed=GENERATOR_SEED, macro_bc=(1, 3, 2, 2, 2), lib=None):
    """The shape of the reference's test scenario: 10x10 quadrilaterals,
    influx segment x in [0, 0.4] on the top (BC 1), free drainage dh/dx = 0
    on the south side (BC 3), no flow elsewhere (src/main.cpp:180-184),
    model_type 3, a full 2x2 Keff(h) table, and an irregularly triangulated
    inclusion of 11x11 nodes in a 0.1 m cell.  macro_bc: the BC types of the
    tags -1 (top segment), -2 (south), -3 (east), -4 (west), -5 (rest of
    the top)."""
    macro = meshgen.macro_unit_square(11, quads=True, segment=(0.0, 0.4))
    micro = meshgen.micro_square_inclusion(11, cell=0.1, side=0.6, jitter=jitter, seed=seed)
    logh = 1.3 - 0.0333 * np.arange(100)
    hh = 10.0 ** logh
    k11 = 0.02 / (1.0 + (0.6 * hh) ** 2.0)
    rows = np.stack([logh, k11, -0.06 * k11, -0.06 * k11, 0.87 * k11], 1)
    p = Problem(macro, micro, rows, 0.64, SOIL_A, SOIL_B, macro_bc=list(macro_bc),
                model_type=3, boundary_flux=boundary_flux, name="fixture10", lib=lib)
    p.options = default_options(lib, AbsTol=1e-6, RelTol=1e-6, MaxKrylov=30)
    p.tend = 0.5
    p.tspan = np.concatenate([[5.0], np.linspace(0.1, 0.5, 5)])
    p.u0 = p.initial_state(-5.0)
    return p


def read_problem_options(path):
    """problem_options.txt exactly as the reference's driver reads it
    (src/main.cpp:32-146): the macro mesh, micro mesh and solution file
    names, h0, tend, no_solns, the no_solns output times, material A (Ksat,
    thetar, thetas, alpha, n), material B, boundary_flux.  A value missing
    at the end of the file leaves the previous one in place, as the
    reference's failed fscanf does (its own test file holds 18 values for
    19 reads, so boundary_flux repeats material B's n)."""
    tok = open(path).read().split()
    if len(tok) < 3:
        raise ValueError("%s: fewer than three file names" % path)
    vals = tok[3:]
    pos = 0
    last = 0.0

    def num():
        nonlocal pos, last
        if pos < len(vals):
            last = float(vals[pos])
        pos += 1
        return last
    h0, tend = num(), num()
    no_solns = int(num())
    tspan = [num() for _ in range(no_solns)]
    soil = []
    for _ in range(2):
        Ks, thr, ths, al, n = (num() for _ in range(5))
        soil.append(dict(Ksat=Ks, thetar=thr, thetas=ths, alpha=al, n=n))
    return dict(macro_mesh_file=tok[0], micro_mesh_file=tok[1], solution_file=tok[2], h0=h0,
                tend=tend, tspan=np.array(tspan), soilA=soil[0], soilB=soil[1],
                boundary_flux=num())


def from_reference_files(options_file, keff_file="Keff.txt", macro_bc=(1, 3, 2, 2, 2),
                         model_type=3):
    """A problem assembled as the reference's main() assembles it
    (src/main.cpp:32-300) from its own input files, read by this library's
    readers: problem_options.txt, the two mesh files it names and the Keff
    table (relative paths are taken from the options file's directory, the
    reference's working directory).  macro_bc and model_type are the values
    main() hard-codes (src/main.cpp:180-192); options are the reference's
    defaults (src/set_exprem_options.cpp:16-26) and u0 = h0 everywhere."""
    import os
    lib = capi.load()
    o = read_problem_options(options_file)
    d = os.path.dirname(os.path.abspath(options_file))
    path = lambda f: f if os.path.isabs(f) else os.path.join(d, f)
    bc = np.ascontiguousarray(macro_bc, dtype=np.int32)
    M, m, K = capi.MacroMesh(), capi.MicroMesh(), capi.Keff()
    check(lib.tsr_macro_mesh_properties(path(o["macro_mesh_file"]).encode(), C.byref(M), ptr(bc)),
          "tsr_macro_mesh_properties")
    check(lib.tsr_micro_mesh_properties(path(o["micro_mesh_file"]).encode(), C.byref(m)),
          "tsr_micro_mesh_properties")
    check(lib.tsr_read_effective_conductivity(path(keff_file).encode(), C.byref(K)),
          "tsr_read_effective_conductivity")
    p = Problem(M, m, K, K.epsilonA, o["soilA"], o["soilB"], macro_bc=list(macro_bc),
                model_type=model_type, boundary_flux=o["boundary_flux"],
                name=os.path.basename(path(o["macro_mesh_file"])))
    p.options = default_options()
    p.tend = o["tend"]
    p.tspan = np.concatenate([[float(len(o["tspan"]))], o["tspan"]])
    p.u0 = np.full(p.N, o["h0"])
    p.h0 = o["h0"]
    p.solution_file = o["solution_file"]
    return p


class Context:
    """The GPU hot path of one problem (a tsr_ctx)."""

    def __init__(self, problem, max_krylov=None, stream=None, gram_schmidt=0):
        """gram_schmidt: 0 modified Gram-Schmidt (the reference's), 1
        classical Gram-Schmidt twice (tsr_set_gram_schmidt)."""
        self.lib = capi.load()
        self.p = problem
        mk = problem.options.MaxKrylov if max_krylov is None else max_krylov
        h = self.lib.tsr_init(C.byref(problem.ud), C.byref(problem.ext), stream, mk)
        if not h:
            raise capi.TsrError(1, "tsr_init")
        self.h = h
        self.N = problem.N
        if gram_schmidt:
            check(self.lib.tsr_set_gram_schmidt(h, gram_schmidt), "tsr_set_gram_schmidt")

    def g(self, u):
        out = np.empty(self.N)
        check(self.lib.tsr_g_eval(self.h, ptr(u), ptr(out)), "tsr_g_eval")
        return out

    def jv(self, u, g0, v, eps):
        out = np.empty(self.N)
        check(self.lib.tsr_jv(self.h, ptr(u), ptr(g0), ptr(v), eps, ptr(out)), "tsr_jv")
        return out

    def water(self, u):
        w = C.c_double()
        check(self.lib.tsr_water_content(self.h, ptr(u), C.byref(w)), "tsr_water_content")
        return w.value

    def autotune(self, u, reps=3):
        """Pick the cell kernel's block size and packing by timing G at u."""
        ms, thr, bud = C.c_double(), C.c_int(), C.c_int()
        check(self.lib.tsr_autotune(self.h, ptr(u), reps, C.byref(ms), C.byref(thr), C.byref(bud)),
              "tsr_autotune")
        return ms.value, thr.value, bud.value

    def dot(self, x, y):
        r = C.c_double()
        check(self.lib.tsr_dot(self.h, ptr(x), ptr(y), x.size, C.byref(r)), "tsr_dot")
        return r.value

    def exprem_step(self, t, u, tspan, solns, opts, stats):
        tt = C.c_double(t)
        check(self.lib.tsr_exprem_step(self.h, C.byref(tt), self.p.tend, ptr(tspan), ptr(solns),
                                       ptr(u), C.byref(opts), C.byref(stats)), "tsr_exprem_step")
        return tt.value

    # ---- ensembles: all scenarios of the context in lockstep
    def load(self, u, t=0.0):
        check(self.lib.tsr_exprem_load(self.h, ptr(u), t), "tsr_exprem_load")

    def store(self):
        u = np.empty(self.N)
        check(self.lib.tsr_exprem_store(self.h, ptr(u)), "tsr_exprem_store")
        return u

    def ensemble_advance(self, stats, tspan=None, solns=None):
        """One accepted step of every scenario short of tend.  stats: a
        ctypes array of S ExpremStats (kept between calls).  Returns
        (t per scenario, status per scenario, number still running)."""
        S = self.p.S
        tspan = np.array([0.0]) if tspan is None else np.ascontiguousarray(tspan, dtype=np.float64)
        t = np.empty(S)
        status = (C.c_int * S)()
        nrun = C.c_int()
        rows = None
        if solns is not None:
            rows = (capi.dp * S)(*[ptr(a) if a is not None else None for a in solns])
        check(self.lib.tsr_ensemble_advance(self.h, self.p.tend, ptr(tspan), rows, C.byref(self.p.options),
                                            stats, ptr(t), status, C.byref(nrun)),
              "tsr_ensemble_advance")
        return t, np.array(status[:]), nrun.value

    def ensemble_water(self, u):
        w = np.empty(self.p.S)
        check(self.lib.tsr_ensemble_water(self.h, ptr(u), ptr(w)), "tsr_ensemble_water")
        return w

    def close(self):
        if self.h:
            self.lib.tsr_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_to_end(step, problem, u0=None, max_steps=100000):
    """The reference driver loop (src/main.cpp:311-341): call one-step
    `step(t, u, tspan, solns, opts, stats) -> t` until t >= tend.  Returns
    (u, tspan_solns, stats, step log)."""
    u = (problem.u0 if u0 is None else u0).copy()
    ns = int(problem.tspan[0])
    solns = np.zeros((ns + 1) * problem.N)
    solns[:problem.N] = u
    stats = capi.ExpremStats()
    t = 0.0
    log = []
    while t < problem.tend and len(log) < max_steps:
        t = step(t, u, problem.tspan, solns, problem.options, stats)
        log.append((stats.NumSteps, t, stats.CurrentStep, stats.CurrentKryDim))
    return u, solns.reshape(ns + 1, problem.N), stats, log
