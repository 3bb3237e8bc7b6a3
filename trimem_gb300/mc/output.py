"""Trajectory output and checkpoints of device chains.

Writers with the interface of the reference's output module
(src/trimem/mc/output/): ``write_points_cells(points, cells)`` appends one
frame, file names are enumerated into parts the same way
(src/trimem/mc/output/_common.py:9-44: ``{stem}.p{n}{suffix}`` with n the
number of parts already present).  Points may be numpy arrays or CUDA
tensors (copied to the host once per frame).

* ``XyzWriter`` — plain-text coordinates, the reference's format
  (src/trimem/mc/output/xyz.py:12-42).
* ``VtuWriter`` — one VTK UnstructuredGrid XML file per frame,
  ``{stem}.{frame}.p{part}.vtu`` as the reference's meshio-based writer
  names them (src/trimem/mc/output/vtu.py:15-43); written here as ASCII
  XML, so it needs no meshio.
* ``save_chain`` / ``load_chain`` — checkpoint of a ``DeviceChain``: the
  positions and the (flipped) half-edge topology with its edge numbering,
  the energy parameters with the
  initial properties and the continuation state, the chain's settings,
  counters and the state of its random generator, so that a loaded chain
  continues bit for bit like the saved one.  The reference's checkpoints
  (XML + HDF5, src/trimem/mc/output/checkpoint.py) need h5py and hold no
  random state; these are a single ``.npz``.
"""
import json
import pathlib
import re

import numpy as np


def _host(points):
    """(N, 3) float64 numpy array from a numpy array or a CUDA tensor."""
    if hasattr(points, "detach"):
        points = points.detach().cpu().numpy()
    return np.asarray(points, dtype=np.float64)


def _create_part(fname):
    """``{stem}.p{n}{suffix}`` with n the number of such files already in
    the directory (src/trimem/mc/output/_common.py:9-44)."""
    fname = pathlib.Path(fname)
    pattern = f"{fname.stem}.p{{}}{fname.suffix}"
    rx = re.compile(re.escape(pattern).replace(r"\{\}", "[0-9]+") + "$")
    parent = fname.parent if str(fname.parent) else pathlib.Path(".")
    n = sum(1 for f in parent.iterdir() if rx.match(f.name)) if parent.exists() else 0
    return fname.with_name(pattern.format(n))


class XyzWriter:
    """Series of point sets in xyz format (all frames in one file)."""

    def __init__(self, fname):
        self.fname = _create_part(pathlib.Path(fname).with_suffix(".xyz"))
        self.step_counter = 0

    def write_points_cells(self, points, cells=None):
        x = _host(points)
        mode = "w" if self.step_counter == 0 else "a"
        with self.fname.open(mode) as fp:
            fp.write(f"{len(x)}\n#\n")
            fp.writelines("C\t{: .6f}\t{: .6f}\t{: .6f}\n".format(*row) for row in x)
        self.step_counter += 1


class VtuWriter:
    """Series of triangle meshes, one VTK UnstructuredGrid file per frame."""

    def __init__(self, fname):
        first = _create_part(pathlib.Path(fname).with_suffix(".0.vtu"))
        self.part = first.suffixes[-2]  # ".p<n>"
        self.prefix = first.name[: -len("".join(first.suffixes))]
        self.dir = first.parent
        self.step = 0

    def write_points_cells(self, points, cells):
        x = _host(points)
        c = np.asarray(cells, dtype=np.int64)
        fname = self.dir / f"{self.prefix}.{self.step}{self.part}.vtu"
        with fname.open("w") as fp:
            fp.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="0.1" '
                     'byte_order="LittleEndian">\n<UnstructuredGrid>\n')
            fp.write(f'<Piece NumberOfPoints="{len(x)}" NumberOfCells="{len(c)}">\n')
            fp.write('<Points>\n<DataArray type="Float64" NumberOfComponents="3" format="ascii">\n')
            fp.writelines("{!r} {!r} {!r}\n".format(*row) for row in x.tolist())
            fp.write("</DataArray>\n</Points>\n<Cells>\n")
            fp.write('<DataArray type="Int64" Name="connectivity" format="ascii">\n')
            fp.writelines(f"{a} {b} {d}\n" for a, b, d in c.tolist())
            fp.write('</DataArray>\n<DataArray type="Int64" Name="offsets" format="ascii">\n')
            fp.write(" ".join(str(3 * (k + 1)) for k in range(len(c))) + "\n")
            fp.write('</DataArray>\n<DataArray type="UInt8" Name="types" format="ascii">\n')
            fp.write(" ".join("5" for _ in range(len(c))) + "\n")  # VTK_TRIANGLE
            fp.write("</DataArray>\n</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
        self.step += 1
        return fname


def read_vtu(fname):
    """(points, cells) of a file written by ``VtuWriter``."""
    import xml.etree.ElementTree as ET

    root = ET.parse(fname).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float64).reshape(-1, 3)
    arrays = {a.get("Name"): a.text for a in piece.findall("Cells/DataArray")}
    cells = np.array(arrays["connectivity"].split(), dtype=np.int64).reshape(-1, 3)
    return pts, cells


_PARAM_FIELDS = ["kappa_b", "kappa_a", "kappa_v", "kappa_c", "kappa_t", "kappa_r", "area_frac", "volume_frac",
                 "curvature_frac", "bond_lc0", "bond_lc1", "bond_a0", "bond_r", "bond_type", "rep_lc1", "rep_r",
                 "n_search", "rlist", "exclusion_level", "cont_delta", "cont_lambda"]
_CHAIN_FIELDS = ["mass", "dt", "L", "T", "flip_ratio", "flip_mode", "flip_batch", "refresh", "seed", "step_index",
                 "accepted", "flips"]


def save_chain(path, chain):
    """Checkpoint of a ``DeviceChain`` (its mesh, energy and state)."""
    x = _host(chain.x)
    faces = chain.mesh.fv_indices()
    topo = chain.mesh.topology()  # half-edge arrays: edge numbering as flipped
    prm = chain.energy.params()
    params = {k: getattr(prm, k) for k in _PARAM_FIELDS}
    state = {k: getattr(chain, k) for k in _CHAIN_FIELDS}
    meta = {"params": params, "chain": state, "rng": chain.rng.bit_generator.state,
            "stencil": getattr(chain.energy, "stencil", 0)}
    np.savez(path, points=x, faces=faces, initial=chain.energy.initial_props(),
             meta=np.array(json.dumps(meta)), **{"he_" + k: v for k, v in topo.items()})


def load_chain(path, stream=None):
    """(chain, mesh, energy) restored from ``save_chain``'s file; the
    positions go to a new CUDA tensor."""
    import torch

    from .. import capi
    from .device import DeviceChain

    with np.load(path, allow_pickle=False) as z:
        x, faces, initial = z["points"], z["faces"], z["initial"]
        meta = json.loads(str(z["meta"]))
        topo = {k[3:]: z[k] for k in z.files if k.startswith("he_")}
    mesh = capi.Mesh(x, faces)
    mesh.set_topology(topo)  # the saved edge numbering (flip proposals pick edges by index)
    energy = capi.Energy(mesh, capi.params(**meta["params"]))
    energy.set_initial_props(initial)
    if meta.get("stencil", 0):
        energy.set_stencil_precision(meta["stencil"])
    c = meta["chain"]
    xt = torch.tensor(x, dtype=torch.float64, device="cuda").contiguous()
    chain = DeviceChain(mesh, energy, xt, mass=c["mass"], dt=c["dt"], n_leapfrog=c["L"], temperature=c["T"],
                        flip_ratio=c["flip_ratio"], flip_mode=c["flip_mode"], flip_batch=c["flip_batch"],
                        refresh=c["refresh"], seed=c["seed"], stream=stream)
    chain.step_index, chain.accepted, chain.flips = c["step_index"], c["accepted"], c["flips"]
    chain.rng.bit_generator.state = meta["rng"]
    return chain, mesh, energy
