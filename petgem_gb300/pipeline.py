"""petgem's pipeline shape on one GPU: Preprocessing -> Solver.setup /
assembly / run -> Postprocessing (petgem/preprocessing.py, solver.py,
postprocessing.py, driven as in kernel.py:32-88).

The stages keep the reference's method names, timer names and inputs (the
params file and PETSc-style KSP options).  Instead of PETSc binary scratch
files, Preprocessing leaves the mesh resident on the GPU (and saves a small
``.npz`` bundle in ``directory_scratch`` so a later process can resume), the
Solver keeps A, b and x as device tensors, and Postprocessing writes the
receiver fields with the reference's HDF5 dataset paths (h5py when
installed, otherwise the same paths as keys of an ``.npz`` file).
"""
import datetime
import os
import platform

import numpy as np
import torch

from . import gmsh
from .common import Print, Timers, parse_petsc_options
from .engine import MU0, DeviceMesh

VERSION = "1.0"
_MESHES = {}      # directory_scratch -> (DeviceMesh, host bundle), same-process stage hand-over


def _mode(inputSetup):
    return inputSetup.model.get("mode")


def _read_array(path):
    """'data' dataset of an HDF5 file (h5py), or a .npy / text file."""
    if path.endswith((".h5", ".hdf5")):
        try:
            import h5py
        except ImportError:
            raise RuntimeError(f"{path}: reading HDF5 needs h5py; provide the array as .npy or text instead")
        with h5py.File(path, "r") as f:
            return np.asarray(f["data"][()])
    if path.endswith(".npy"):
        return np.load(path)
    return np.loadtxt(path)


class Preprocessing:
    """Mesh import, topology / DOF numbering / boundaries on the GPU
    (petgem/preprocessing.py:40-538)."""

    def run(self, inputSetup):
        Timers()["Preprocessing"].start()
        model, run, output = inputSetup.model, inputSetup.run, inputSetup.output
        mode = _mode(inputSetup)
        if mode != "csem":
            raise NotImplementedError("MT mode: the plane-wave boundary RHS (petgem/solver.py:318-512) is not "
                                      "built on the GPU yet; CSEM is supported")
        data_model = model[mode]
        p = int(run["nord"])
        mesh = gmsh.read(model["mesh"])
        if run.get("conductivity_from_file"):
            sigma = np.asarray(_read_array(data_model["sigma"]["file"]), dtype=np.float64)
        else:
            phys = mesh.physical - 1                           # 0-based (preprocessing.py:262)
            sh = np.asarray(data_model["sigma"]["horizontal"], dtype=np.float64)
            sv = np.asarray(data_model["sigma"]["vertical"], dtype=np.float64)
            sigma = np.stack([sh[phys], sv[phys]], axis=1)
        receivers = np.atleast_2d(np.asarray(_read_array(model["receivers"]), dtype=np.float64))
        dm = DeviceMesh(mesh.points, mesh.tets, p)
        src = dict(data_model["source"])
        src_elem = dm.locate_source(src)
        if int(src_elem.item()) < 0:
            raise ValueError("Source no located in the computational domain. Please, verify source position or "
                             "improve the mesh quality.")
        bundle = {"nodes": mesh.points, "tets": mesh.tets, "sigma": sigma, "receivers": receivers, "nord": p}
        np.savez(os.path.join(output["directory_scratch"], "gb300_preprocessing.npz"), **bundle)
        _MESHES[output["directory_scratch"]] = (dm, bundle)
        Print.master(f"     Number of elements: {dm.T}")
        Print.master(f"     Number of faces:    {dm.nF}")
        Print.master(f"     Number of edges:    {dm.nE}")
        Print.master(f"     Number of dofs:     {dm.N}")
        Print.master(f"     Number of boundaries: {dm.bnd.numel()}")
        Timers()["Preprocessing"].stop()


class Solver:
    """Assembly and Krylov solve (petgem/solver.py:31-598)."""

    def setup(self, inputSetup):
        Timers()["Setup"].start()
        scratch = inputSetup.output["directory_scratch"]
        if scratch in _MESHES:
            self.mesh, self.bundle = _MESHES[scratch]
        else:
            d = np.load(os.path.join(scratch, "gb300_preprocessing.npz"))
            self.bundle = {k: d[k] for k in d.files}
            self.mesh = DeviceMesh(self.bundle["nodes"], self.bundle["tets"], int(self.bundle["nord"]))
            _MESHES[scratch] = (self.mesh, self.bundle)
        self.total_num_dofs = self.mesh.N
        self.boundaries = self.mesh.bnd
        Timers()["Setup"].stop()

    def assembly(self, inputSetup):
        Timers()["Assembly"].start()
        data_model = inputSetup.model[_mode(inputSetup)]
        src = dict(data_model["source"])
        freq = float(src["frequency"])
        m = self.mesh
        self.A = m.assemble(self.bundle["sigma"], freq, fused=True)
        self.b = [torch.zeros(m.N, dtype=torch.complex128, device=m.device)]
        self.x = [torch.zeros_like(self.b[0])]
        m.source_vector(src, self.b[0])
        torch.cuda.synchronize()
        Timers()["Assembly"].stop()

    def run(self, inputSetup, options=None):
        """PEC + KSP solve.  options: dict from parse_petsc_options (petgem
        reads them from the PETSc options database, solver.py:588)."""
        opts = options or {}
        Timers()["SetBoundaries"].start()
        self.mesh.apply_pec(self.A, self.b[0])
        torch.cuda.synchronize()
        Timers()["SetBoundaries"].stop()
        Timers()["Solver"].start()
        ksp = str(opts.get("ksp_type", "gmres"))
        if ksp not in ("gmres", "cocg"):
            raise ValueError(f"-ksp_type {ksp}: supported types are gmres and cocg")
        pc = str(opts.get("pc_type", "jacobi"))
        if pc not in ("jacobi", "sor", "none", "bjacobi"):
            raise ValueError(f"-pc_type {pc}: supported preconditioner is jacobi")
        self.info = []
        for i in range(len(self.b)):
            x, info = self.mesh.solve(self.A, self.b[i], rtol=float(opts.get("ksp_rtol", 1e-8)),
                                      restart=int(opts.get("ksp_gmres_restart", 30)),
                                      max_it=int(opts.get("ksp_max_it", 10000)),
                                      precision=str(opts.get("pg_precision", "fp64")), ksp=ksp,
                                      raise_on_fail=False)
            self.x[i] = x
            self.info.append(info)
            Print.master(f"     KSP {ksp}: {info.iterations} iterations, true relative residual {info.relres:.3e}")
            np.save(os.path.join(inputSetup.output["directory_scratch"], f"x{i}.npy"), x.cpu().numpy())
        Timers()["Solver"].stop()


class Postprocessing:
    """Receiver interpolation and output (petgem/postprocessing.py:42-476)."""

    def run(self, inputSetup, solver=None):
        Timers()["Postprocessing"].start()
        model, run, output = inputSetup.model, inputSetup.run, inputSetup.output
        mode = _mode(inputSetup)
        scratch = output["directory_scratch"]
        if solver is not None:
            m, xs, bundle = solver.mesh, solver.x, solver.bundle
        else:
            m, bundle = _MESHES[scratch]
            xs = [torch.as_tensor(np.load(os.path.join(scratch, "x0.npy")), device=m.device)]
        freq = float(model[mode]["source"]["frequency"])
        fields, keep = m.receiver_fields(xs[0], bundle["receivers"], freq)
        dropped = np.nonzero(~keep.cpu().numpy())[0]
        if dropped.size:
            Print.master("        The following receivers were not located and will not be taken into account "
                         + str(dropped))
        F = fields.cpu().numpy()
        self.fields = F
        elapsed = Timers()["Assembly"].elapsed + Timers()["Solver"].elapsed
        out = {
            "machine/machine": f"{platform.uname().node}. {platform.uname().release}. {platform.uname().processor}",
            "machine/num_processors": 1,
            "machine/petgem_version": VERSION,
            "model/date": datetime.datetime.today().isoformat(),
            "model/mesh_file": str(model["mesh"]),
            "model/receivers_file": str(model["receivers"]),
            "model/nord": int(run["nord"]),
            "model/dof": int(m.N),
            "model/cuda": bool(run.get("cuda", False)),
            "model/vtk": bool(output.get("vtk", False)),
            "model/mode": mode,
            "model/num-polarizations": int(run["num_polarizations"]),
            "model/solver": str(getattr(solver, "ksp", "gmres")) if solver else "gmres",
            "model/run-time (s)": float(elapsed),
            "model/frequency (Hz)": freq,
            "model/E-fields/x": F[:, 0], "model/E-fields/y": F[:, 1], "model/E-fields/z": F[:, 2],
            "model/H-fields/x": F[:, 3], "model/H-fields/y": F[:, 4], "model/H-fields/z": F[:, 5],
        }
        src = model[mode]["source"]
        if run.get("conductivity_from_file"):
            out["model/sigma-file"] = str(model[mode]["sigma"]["file"])
        else:
            out["model/sigma_horizontal (S/m)"] = np.asarray(model[mode]["sigma"]["horizontal"], dtype=np.float64)
            out["model/sigma_vertical (S/m)"] = np.asarray(model[mode]["sigma"]["vertical"], dtype=np.float64)
        out["model/source_position (m)"] = np.asarray(src["position"], dtype=np.float64)
        out["model/source_azimuth (deg)"] = src["azimuth"]
        out["model/source_dip (deg)"] = src["dip"]
        out["model/source_current (Am)"] = src["current"]
        out["model/source_length (m)"] = src["length"]
        name = f"{mode}_petgemV{VERSION}_{datetime.datetime.today().strftime('%Y-%m-%d')}"
        self.output_file = write_results(os.path.join(output["directory"], name), out)
        Timers()["Postprocessing"].stop()
        return F


def write_results(stem, datasets):
    """HDF5 with petgem's group/dataset paths (postprocessing.py:341-461) when
    h5py is installed, else an .npz whose keys are those paths."""
    try:
        import h5py
    except ImportError:
        path = stem + ".npz"
        np.savez(path, **{k: np.asarray(v) for k, v in datasets.items()})
        return path
    path = stem + ".h5"
    with h5py.File(path, "w") as f:
        for k, v in datasets.items():
            f.create_dataset(k, data=v)
    return path


def fieldInterpolator(solution_vector, nodes, elemsN, elemsE, edgesN, elemsF, facesE, dof_connectivity, points,
                      inputSetup):
    """petgem/postprocessing.py:479: E and H at points; receivers outside
    the mesh are dropped.  The topology arguments are recomputed on the GPU
    (bit-exact with the ones petgem passes)."""
    p = int(inputSetup.run["nord"])
    mode = _mode(inputSetup)
    freq = float(inputSetup.model[mode]["source"]["frequency"]) if mode == "csem" else \
        float(inputSetup.model[mode]["frequency"])
    m = DeviceMesh(nodes, elemsN, p, pattern=False)
    x = solution_vector
    if not torch.is_tensor(x):
        x = torch.as_tensor(np.asarray(x, dtype=np.complex128))
    F, _ = m.receiver_fields(x.to(m.device).contiguous(), points, freq)
    return F.cpu().numpy()


def run_kernel(params_path, argv=()):
    """The driver of petgem's kernel.py:32-88 on one GPU."""
    from .common import InputParameters
    opts = parse_petsc_options(list(argv))
    setup = InputParameters(params_path)
    Print.header()
    Print.master("  Data preprocessing")
    Preprocessing().run(setup)
    Print.master("  Run modelling")
    solver = Solver()
    solver.setup(setup)
    solver.assembly(setup)
    solver.run(setup, opts)
    Print.master("  Data postprocessing")
    post = Postprocessing()
    post.run(setup, solver)
    return setup, solver, post
