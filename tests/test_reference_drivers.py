"""The reference's own Python drivers run unchanged over trimem_gb300.core.

trimem's Monte Carlo layer (``trimem.mc``: hmc.py, mesh.py, evaluators.py,
config.py, util.py, app.py) reaches native code only through
``from .. import core as m``.  A user switches it to this library by mapping
``trimem.core`` to ``trimem_gb300.core`` before importing ``trimem.mc``;
these tests do exactly that with the reference's sources, unmodified, and
check what they compute against the oracle.

The reference is not part of this repository: its sources are loaded from
the folder named by the environment variable TRIMEM_REFERENCE (the root of a
trimem checkout, holding ``src/trimem``) and the tests skip when it is
unset.  h5py and meshio, which the reference's output package imports at
module level, are replaced by empty stand-in modules when they are not
installed; the runs write xyz output and keep their checkpoints in memory.
"""
import importlib
import importlib.util
import io
import os
import sys
import types

import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

REF = os.environ.get("TRIMEM_REFERENCE")


def load_reference_trimem():
    """The reference's ``trimem`` package with ``trimem.core`` mapped to
    ``trimem_gb300.core``; skips when TRIMEM_REFERENCE is unset."""
    if not REF:
        pytest.skip("TRIMEM_REFERENCE (root of a trimem checkout) is not set")
    src = os.path.join(REF, "src", "trimem")
    if not os.path.isfile(os.path.join(src, "mc", "hmc.py")):
        pytest.skip(f"no trimem sources under {REF}")
    from trimem_gb300 import load_core

    core = load_core()
    for name in [k for k in sys.modules if k == "trimem" or k.startswith("trimem.")]:
        del sys.modules[name]
    for missing in ("h5py", "meshio"):
        try:
            importlib.import_module(missing)
        except ImportError:
            sys.modules[missing] = types.ModuleType(missing)
    spec = importlib.util.spec_from_file_location("trimem", os.path.join(src, "__init__.py"),
                                                  submodule_search_locations=[src])
    pkg = importlib.util.module_from_spec(spec)
    sys.modules["trimem"] = pkg
    spec.loader.exec_module(pkg)
    sys.modules["trimem.core"] = core
    pkg.core = core
    return pkg


def energy_params(core, prm):
    """core.EnergyParams from a parameter dict of the workloads."""
    ep = core.EnergyParams()
    for k in ("kappa_b", "kappa_a", "kappa_v", "kappa_c", "kappa_t", "kappa_r", "area_frac", "volume_frac",
              "curvature_frac"):
        setattr(ep, k, prm[k])
    bp = ep.bond_params
    bp.lc0, bp.lc1, bp.a0, bp.r = prm["bond_lc0"], prm["bond_lc1"], prm["bond_a0"], prm["bond_r"]
    bp.type = core.BondType.Edge if prm["bond_type"] == 0 else core.BondType.Area
    ep.bond_params = bp
    rp = ep.repulse_params
    rp.lc1, rp.r, rp.rlist, rp.exclusion_level = prm["rep_lc1"], prm["rep_r"], prm["rlist"], prm["exclusion_level"]
    rp.n_search = "cell-list" if prm["n_search"] == 0 else "verlet-list"
    ep.repulse_params = rp
    cp = ep.continuation_params
    cp.delta, cp.lam = prm["cont_delta"], prm["cont_lambda"]
    ep.continuation_params = cp
    return ep


def test_reference_hmc_reproduces_its_golden_chain():
    """The reference's HMC class (pure numpy) on its own golden chain, with
    the package imported over this library's core."""
    import json

    trimem = load_reference_trimem()
    from trimem.mc.hmc import HMC

    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "hmc_icosahedron.json")))
    np.random.seed(42)
    h = HMC(np.array(g["x0"]), lambda x: 0.5 * x.ravel().dot(x.ravel()), lambda x: x,
            options={"info_step": 10, "time_step": 1.0e-1})
    h.run(10)
    assert trimem.core.__name__.startswith("trimem_gb300")
    assert np.linalg.norm(h.x - np.array(g["ref_hmc"])) < 1.0e-14


@pytest.mark.gpu
def test_reference_mesh_hmc_matches_the_oracle_chain(built):
    """MeshHMC driven by EnergyEvaluators.fun/grad over this library's
    EnergyManager follows the oracle's HMC chain (same numpy random stream,
    the oracle's energy and gradient) step for step."""
    from oracle import oracle as O

    trimem = load_reference_trimem()
    core = trimem.core
    from trimem.mc.evaluators import EnergyEvaluators
    from trimem.mc.hmc import MeshHMC, get_step_counters
    from trimem.mc.mesh import Mesh

    p, f = meshgen.jittered_icosphere(3, seed=3)
    prm = dict(workload_params(p, f, excl=1, rep_scale=1.2), cont_lambda=0.0)
    mesh = Mesh(p.copy(), f)
    estore = core.EnergyManager(mesh.trimesh, energy_params(core, prm))
    funcs = EnergyEvaluators(mesh, estore, None, {"info_step": 0, "output_step": 0, "refresh_step": 1})
    opts = {"time_step": 2e-6, "num_integration_steps": 10, "info_step": 0}
    np.random.seed(7)
    hmc = MeshHMC(mesh, funcs.fun, funcs.grad, counter=get_step_counters(), options=opts)
    hmc.run(12)

    mo = O.Mesh(p.copy(), f)
    eo = O.Energy(mo, O.default_params(**prm))
    pts = mo.points()

    def fun(x):
        pts[:] = x
        return eo.energy(mo)

    def grad(x):
        pts[:] = x
        return eo.gradient(mo)

    np.random.seed(7)
    x_or, acc = O.hmc_chain(p.copy(), fun, grad, n_steps=12, dt=opts["time_step"], n_leapfrog=10)
    assert 0 < acc
    assert np.array_equal(mesh.x, hmc.x)
    rel = np.linalg.norm(hmc.x - x_or) / np.linalg.norm(x_or)
    assert rel < 1e-10, rel


@pytest.mark.gpu
def test_reference_monte_carlo_with_flips(built):
    """MeshMonteCarlo (HMC moves and serial / parallel flip sweeps, the
    evaluators' callback refreshing the neighbour list and advancing the
    continuation) over this library: the final mesh is valid and its
    properties equal the oracle's at the same state."""
    from oracle import oracle as O

    trimem = load_reference_trimem()
    core = trimem.core
    from trimem.mc.evaluators import EnergyEvaluators
    from trimem.mc.hmc import MeshFlips, MeshHMC, MeshMonteCarlo, get_step_counters
    from trimem.mc.mesh import Mesh

    p, f = meshgen.jittered_icosphere(3, seed=5)
    prm = workload_params(p, f, excl=2, rep_scale=1.2)
    prm.update(cont_delta=0.05, cont_lambda=0.5)
    for flip_type in ("serial", "parallel"):
        mesh = Mesh(p.copy(), f)
        estore = core.EnergyManager(mesh.trimesh, energy_params(core, prm))
        funcs = EnergyEvaluators(mesh, estore, None, {"info_step": 0, "output_step": 0, "refresh_step": 2})
        counter = get_step_counters()
        np.random.seed(11)
        hmc = MeshHMC(mesh, funcs.fun, funcs.grad, counter=counter,
                      options={"time_step": 2e-6, "num_integration_steps": 10, "info_step": 0})
        flips = MeshFlips(mesh, estore, counter=counter,
                          options={"flip_type": flip_type, "flip_ratio": 0.3, "info_step": 0})
        mmc = MeshMonteCarlo(hmc, flips, counter=counter, callback=funcs.callback)
        mmc.run(30)
        assert counter["move"] + counter["flip"] == 30 and counter["flip"] > 0, (flip_type, counter)
        assert mesh.trimesh.check() == 0
        assert estore.eparams.continuation_params.lam > 0.5
        fv = mesh.f
        assert len(np.unique(np.sort(fv, axis=1), axis=0)) == len(fv)
        # properties of the final state against the oracle on the same
        # positions and faces, neighbour list rebuilt at that state
        estore.update_repulsion(mesh.trimesh)
        vp = estore.properties(mesh.trimesh)
        mo = O.Mesh(np.array(mesh.x), np.array(fv))
        eo = O.Energy(mo, O.default_params(**prm))
        ref = eo.properties(mo)
        got = [vp.area, vp.volume, vp.curvature, vp.bending, vp.tethering, vp.repulsion]
        for k, (a, b) in enumerate(zip(got, ref)):
            assert abs(a - b) <= 1e-10 * max(abs(b), 1e-300), (flip_type, k, a, b)


@pytest.mark.gpu
def test_reference_mc_app_runs_minimise_then_hmc_restart(built, tmp_path, monkeypatch, capsys):
    """The reference's command-line layer (mc_app config / run; util.run,
    run_minim, run_mc) over this library: default config written by the
    reference, a minimisation from an STL file, then an HMC run restarted
    from the minimisation's checkpoint.  Checkpoints are kept in memory (the
    reference writes them with h5py, which is not installed); output is xyz."""
    trimem = load_reference_trimem()
    core = trimem.core
    from trimem.mc import app, util

    # the input geometry, written as ASCII STL
    p, f = meshgen.icosphere(3)
    stl = tmp_path / "inp.stl"
    with open(stl, "w") as fh:
        fh.write("solid inp\n")
        for a, b, c in f:
            n = np.cross(p[b] - p[a], p[c] - p[a])
            n /= np.linalg.norm(n)
            fh.write(f"facet normal {n[0]:.17g} {n[1]:.17g} {n[2]:.17g}\n outer loop\n")
            for v in (a, b, c):
                fh.write(f"  vertex {p[v][0]:.17g} {p[v][1]:.17g} {p[v][2]:.17g}\n")
            fh.write(" endloop\nendfacet\n")
        fh.write("endsolid inp\n")
    assert core.read_mesh(str(stl)).n_vertices() == len(p)

    checkpoints = {}

    class MemoryCheckpointWriter:
        def __init__(self, prefix):
            self.fname = f"{prefix}.{len(checkpoints.get(prefix, []))}.cpt"
            self.prefix = prefix

        def write(self, points, cells, config):
            buf = io.StringIO()
            config.write(buf)
            checkpoints.setdefault(self.prefix, []).append((np.array(points), np.array(cells), buf.getvalue()))

    class MemoryCheckpointReader:
        def __init__(self, prefix, num):
            self.prefix, self.num = prefix, num
            self.fname = f"{prefix}.{num}.cpt"

        def read(self):
            import configparser

            pts, cells, text = checkpoints[self.prefix][self.num]
            conf = configparser.ConfigParser(inline_comment_prefixes=("#", ";"))
            conf.read_string(text)
            return pts, cells, conf

    monkeypatch.setattr(util, "CheckpointWriter", MemoryCheckpointWriter)
    monkeypatch.setattr(util, "CheckpointReader", MemoryCheckpointReader)

    conf = tmp_path / "inp.conf"
    monkeypatch.setattr(sys, "argv", ["mc_app", "config", "--strip", "--conf", str(conf)])
    app.cli()
    text = conf.read_text()
    settings = {"output_format": "xyz", "algorithm": "minimize", "step_size": "1.0e-5"}
    lines = []
    for line in text.splitlines():
        key = line.split("=")[0].strip()
        if key in settings and "=" in line:
            line = f"{key} = {settings[key]}"
        lines.append(line)
    conf.write_text("\n".join(lines) + "\n")
    cfg = trimem.mc.config.read_config(conf)
    mesh0 = trimem.mc.mesh.read_trimesh(str(stl))
    estore0, _ = util.setup_energy_manager(cfg)
    e0 = estore0.energy(mesh0.trimesh)

    monkeypatch.setattr(sys, "argv", ["mc_app", "run", "--conf", str(conf)])
    app.cli()
    prefix = str(conf.with_suffix(""))
    assert len(checkpoints[prefix]) == 1
    x_min, f_min, _ = checkpoints[prefix][0]
    m1 = core.TriMesh(x_min, f_min)
    estore1, _ = util.setup_energy_manager(cfg)
    e1 = estore1.energy(m1)
    assert e1 < e0, (e1, e0)

    # HMC restarted from the minimisation's checkpoint
    conf.write_text(conf.read_text().replace("algorithm = minimize", "algorithm = hmc"))
    monkeypatch.setattr(sys, "argv", ["mc_app", "run", "--conf", str(conf), "--restart", "0"])
    app.cli()
    assert len(checkpoints[prefix]) == 2
    x_hmc, f_hmc, text_hmc = checkpoints[prefix][1]
    assert x_hmc.shape == x_min.shape and np.isfinite(x_hmc).all()
    assert core.TriMesh(x_hmc, f_hmc).check() == 0
    assert '"move"' in text_hmc and '"flip"' in text_hmc
    assert any(tmp_path.glob("inp*.xyz"))  # the trajectory, every 10th step
    captured = capsys.readouterr().out
    assert "Minimization finished" in captured and "HMC-Step" in captured
