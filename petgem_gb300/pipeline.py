"""petgem's pipeline shape on one GPU: Preprocessing -> Solver.setup /
assembly / run -> Postprocessing (petgem/preprocessing.py, solver.py,
postprocessing.py, driven as in kernel.py:32-88).

The stages keep the reference's method names, timer names and inputs (the
params file and PETSc-style KSP options).  Instead of PETSc binary scratch
files, Preprocessing leaves the mesh resident on the GPU (and saves a small
``.npz`` bundle in ``directory_scratch`` so a later process can resume), the
Solver keeps A, b and x as device tensors (and writes x{i}.dat in petgem's
PETSc binary format; it also starts from petgem's own preprocessing scratch
files when those are what the scratch directory holds), and Postprocessing writes the
receiver fields with the reference's HDF5 dataset paths (h5py when
installed, otherwise the same paths as keys of an ``.npz`` file).
"""
import datetime
import os
import platform

import numpy as np
import torch

from . import gmsh, petsc_io
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
        if mode == "csem":
            src = dict(data_model["source"])
            src_elem = dm.locate_source(src)
            if int(src_elem.item()) < 0:
                raise ValueError("Source no located in the computational domain. Please, verify source position or "
                                 "improve the mesh quality.")
        else:
            dm.mt_boundary()           # boundary faces, box sides (preprocessing.py:314-381)
        bundle = {"nodes": mesh.points, "tets": mesh.tets, "sigma": sigma, "receivers": receivers, "nord": p}
        np.savez(os.path.join(output["directory_scratch"], "gb300_preprocessing.npz"), **bundle)
        _MESHES[output["directory_scratch"]] = (dm, bundle)
        Print.master(f"     Number of elements: {dm.T}")
        Print.master(f"     Number of faces:    {dm.nF}")
        Print.master(f"     Number of edges:    {dm.nE}")
        Print.master(f"     Number of dofs:     {dm.N}")
        Print.master(f"     Number of boundaries: {dm.bnd.numel()}")
        Timers()["Preprocessing"].stop()


def ksp_settings(opts, nord):
    """(ksp, precond) for the solver from the PETSc options petgem's
    KSPSolve reads (petgem/solver.py:584-594): -ksp_type gmres | cocg,
    -pc_type jacobi | bjacobi | sor | none | hypre (-pc_hypre_type ams).
    bjacobi: one block per edge / face / element; sor (petgem's default, a
    sequential sweep) and none run with the entity blocks as well; hypre's
    AMS (auxiliary-space Maxwell) is served by its one-level relative, Jacobi
    plus one Jacobi step on the discrete gradients and (nord >= 2) on the
    vector P1 fields, built for nord <= 3.  Anything else raises ValueError."""
    ksp = str(opts.get("ksp_type", "gmres"))
    if ksp not in ("gmres", "cocg"):
        raise ValueError(f"-ksp_type {ksp}: supported types are gmres and cocg")
    pc = str(opts.get("pc_type", "jacobi"))
    if pc not in ("jacobi", "sor", "none", "bjacobi", "hypre"):
        raise ValueError(f"-pc_type {pc}: supported preconditioners are jacobi, bjacobi and hypre (ams)")
    if pc == "hypre" and str(opts.get("pc_hypre_type", "ams")) != "ams":
        raise ValueError("-pc_type hypre: supported -pc_hypre_type is ams")
    precond = {"jacobi": "jacobi", "hypre": "grad"}.get(pc, "block")
    if precond == "grad" and int(nord) > 3:
        raise ValueError("-pc_type hypre: the gradient correction is built for nord <= 3")
    return ksp, precond


class Solver:
    """Assembly and Krylov solve (petgem/solver.py:31-598)."""

    def setup(self, inputSetup):
        Timers()["Setup"].start()
        scratch = inputSetup.output["directory_scratch"]
        if scratch in _MESHES:
            self.mesh, self.bundle = _MESHES[scratch]
        elif os.path.exists(os.path.join(scratch, "gb300_preprocessing.npz")):
            d = np.load(os.path.join(scratch, "gb300_preprocessing.npz"))
            self.bundle = {k: d[k] for k in d.files}
            self.mesh = DeviceMesh(self.bundle["nodes"], self.bundle["tets"], int(self.bundle["nord"]))
            _MESHES[scratch] = (self.mesh, self.bundle)
        else:
            # scratch written by petgem's own Preprocessing (PETSc binary files)
            nodes, tets, sigma = petsc_io.read_petgem_scratch(scratch)
            receivers = np.atleast_2d(np.asarray(_read_array(inputSetup.model["receivers"]), dtype=np.float64))
            p = int(inputSetup.run["nord"])
            self.bundle = {"nodes": nodes, "tets": tets, "sigma": sigma, "receivers": receivers, "nord": p}
            self.mesh = DeviceMesh(nodes, tets, p)
            _MESHES[scratch] = (self.mesh, self.bundle)
        self.total_num_dofs = self.mesh.N
        self.boundaries = self.mesh.bnd
        Timers()["Setup"].stop()

    def assembly(self, inputSetup):
        Timers()["Assembly"].start()
        mode = _mode(inputSetup)
        data_model = inputSetup.model[mode]
        m = self.mesh
        self.mode = mode
        if mode == "csem":
            src = dict(data_model["source"])
            freq = float(src["frequency"])
            self.A = m.assemble(self.bundle["sigma"], freq, fused=True)
            self.b = [torch.zeros(m.N, dtype=torch.complex128, device=m.device)]
            m.source_vector(src, self.b[0])
        else:
            # MT: no PEC; one plane-wave RHS per polarisation (solver.py:318-512)
            freq = float(data_model["frequency"])
            self.polarizations = [str(q) for q in data_model["polarization"]]
            self.A = m.assemble(self.bundle["sigma"], freq, fused=True)
            B = m.mt_rhs(self.bundle["sigma"], freq, self.polarizations)
            self.b = [B[:, k].contiguous() for k in range(B.shape[1])]
        self.x = [torch.zeros_like(bk) for bk in self.b]
        torch.cuda.synchronize()
        Timers()["Assembly"].stop()

    def run(self, inputSetup, options=None):
        """PEC + KSP solve.  options: dict from parse_petsc_options (petgem
        reads them from the PETSc options database, solver.py:588)."""
        opts = options or {}
        if getattr(self, "mode", "csem") == "csem":
            Timers()["SetBoundaries"].start()
            self.mesh.apply_pec(self.A, self.b[0])
            torch.cuda.synchronize()
            Timers()["SetBoundaries"].stop()
        Timers()["Solver"].start()
        ksp, precond = ksp_settings(opts, self.mesh.p)
        self.info = []
        self.ksp = ksp
        # all polarisations in one batched solve (one SpMM per iteration)
        B = torch.stack(self.b, dim=1).contiguous() if len(self.b) > 1 else self.b[0]
        X, info = self.mesh.solve(self.A, B, rtol=float(opts.get("ksp_rtol", 1e-8)),
                                  restart=int(opts.get("ksp_gmres_restart", 30)),
                                  max_it=int(opts.get("ksp_max_it", 10000)),
                                  precision=str(opts.get("pg_precision", "fp64")), ksp=ksp,
                                  raise_on_fail=False, precond=precond, pec=getattr(self, "mode", "csem") == "csem")
        for i in range(len(self.b)):
            self.x[i] = X[:, i].contiguous() if X.ndim == 2 else X
            self.info.append(info)
            Print.master(f"     KSP {ksp}: {info.iterations} iterations, true relative residual "
                         f"{info.relres_per_rhs[i] if info.relres_per_rhs is not None else info.relres:.3e}")
            # x{i}.dat as petgem's Solver writes it (PETSc binary), readable by petgem's Postprocessing
            petsc_io.write_vec(os.path.join(inputSetup.output["directory_scratch"], f"x{i}.dat"),
                               self.x[i].cpu().numpy())
        Timers()["Solver"].stop()


class Postprocessing:
    """Receiver interpolation and output (petgem/postprocessing.py:42-476)."""

    def run(self, inputSetup, solver=None):
        Timers()["Postprocessing"].start()
        model, run, output = inputSetup.model, inputSetup.run, inputSetup.output
        mode = _mode(inputSetup)
        scratch = output["directory_scratch"]
        npol = int(run["num_polarizations"])
        if solver is not None:
            m, xs, bundle = solver.mesh, solver.x, solver.bundle
        else:
            m, bundle = _MESHES[scratch]
            xs = [torch.as_tensor(petsc_io.read_vec(os.path.join(scratch, f"x{i}.dat")), device=m.device)
                  for i in range(npol)]
        freq = float(model[mode]["source"]["frequency"]) if mode == "csem" else float(model[mode]["frequency"])
        Fs = []
        for x in xs:
            fields, keep = m.receiver_fields(x, bundle["receivers"], freq)
            Fs.append(fields.cpu().numpy())
        dropped = np.nonzero(~keep.cpu().numpy())[0]
        if dropped.size:
            Print.master("        The following receivers were not located and will not be taken into account "
                         + str(dropped))
        F = Fs[0]
        self.fields = F if mode == "csem" else Fs
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
            "model/num-polarizations": npol,
            "model/solver": str(getattr(solver, "ksp", "gmres")) if solver else "gmres",
            "model/run-time (s)": float(elapsed),
        }
        if run.get("conductivity_from_file"):
            out["model/sigma-file"] = str(model[mode]["sigma"]["file"])
        else:
            out["model/sigma_horizontal (S/m)"] = np.asarray(model[mode]["sigma"]["horizontal"], dtype=np.float64)
            out["model/sigma_vertical (S/m)"] = np.asarray(model[mode]["sigma"]["vertical"], dtype=np.float64)
        out["model/frequency (Hz)"] = freq
        if mode == "csem":
            src = model[mode]["source"]
            out["model/source_position (m)"] = np.asarray(src["position"], dtype=np.float64)
            out["model/source_azimuth (deg)"] = src["azimuth"]
            out["model/source_dip (deg)"] = src["dip"]
            out["model/source_current (Am)"] = src["current"]
            out["model/source_length (m)"] = src["length"]
            for c, k in enumerate("xyz"):
                out[f"model/E-fields/{k}"] = F[:, c]
                out[f"model/H-fields/{k}"] = F[:, 3 + c]
        else:
            pols = [str(q) for q in model[mode]["polarization"]]
            out["model/polarization"] = np.asarray(pols)
            for i, q in enumerate(pols):
                for c, k in enumerate("xyz"):
                    out[f"model/E-fields_mode_{q}/{k}"] = Fs[i][:, c]
                    out[f"model/H-fields_mode_{q}/{k}"] = Fs[i][:, 3 + c]
            if npol == 2:
                rho, phase, tip, Z = computeImpedance(Fs, 2.0 * np.pi * freq, MU0)
                self.impedance, self.apparent_resistivity, self.phase, self.tipper = Z, rho, phase, tip
                for j, k in enumerate(("xx", "xy", "yx", "yy")):
                    out[f"model/impedance/{k}"] = Z[j]
                    out[f"model/apparent_resistivity/{k}"] = rho[j]
                    out[f"model/phase/{k}"] = phase[j]
                out["model/tipper/x"], out["model/tipper/y"] = tip[0], tip[1]
        name = f"{mode}_petgemV{VERSION}_{datetime.datetime.today().strftime('%Y-%m-%d')}"
        if output.get("vtk"):
            self.vtk_file = write_vtk_fields(m, xs, bundle, mode, model[mode], freq,
                                             os.path.join(output["directory"], name + ".vtk"))
        self.output_file = write_results(os.path.join(output["directory"], name), out)
        Timers()["Postprocessing"].stop()
        return F if mode == "csem" else Fs


def write_vtk_fields(m, xs, bundle, mode, data_model, freq, path):
    """Nodal E and H (GPU node averaging) and the conductivity as a VTK file
    with petgem's array names (postprocessing.py:173-336); petgem stores the
    horizontal conductivity in both cell arrays, and so does this file."""
    from . import vtk
    pd = {}
    if mode == "csem":
        tags = [""]
    else:
        pols = [str(q) for q in data_model["polarization"]]
        tags = ["_mode" + q for q in pols]
    for x, tag in zip(xs, tags):
        F = m.node_fields(x, freq).cpu().numpy()
        for c, name in enumerate(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
            pd[f"{mode}_{name}_real{tag}"] = F[:, c].real
        for c, name in enumerate(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
            pd[f"{mode}_{name}_imag{tag}"] = F[:, c].imag
    sigma = np.asarray(bundle["sigma"], dtype=np.float64)
    cd = {"sigma_horizontal": sigma[:, 0], "sigma_vertical": sigma[:, 0]}
    vtk.write(path, bundle["nodes"], bundle["tets"], pd, cd)
    return path


def computeImpedance(fields, omega, mu):
    """Apparent resistivity, phase, tipper and impedance from two
    polarisations' receiver fields (R, 6) each (petgem/postprocessing.py:619-688):
    Z solves E = Z H per receiver, rho_a = |Z|^2 / (omega mu), phase =
    atan(-Im Z / Re Z) in degrees mod 360, and the tipper T solves
    Hz = Tx Hx + Ty Hy.  Returns ([rho xx, xy, yx, yy], [phase ...], [Tx, Ty],
    [Z xx, xy, yx, yy])."""
    f1, f2 = np.asarray(fields[0]), np.asarray(fields[1])
    e1x, e1y, h1x, h1y, h1z = f1[:, 0], f1[:, 1], f1[:, 3], f1[:, 4], f1[:, 5]
    e2x, e2y, h2x, h2y, h2z = f2[:, 0], f2[:, 1], f2[:, 3], f2[:, 4], f2[:, 5]
    # Cramer's rule on the two polarisations, in the reference's factorisation
    m1 = h2y * h2x * h1y - h2y * h2y * h1x
    m2 = h2x * h2x * h1y - h2y * h2x * h1x
    m3 = e2x * h2x * h1y - h2y * e2x * h1x
    m4 = h2y * e2y * h1y - h2y * h2y * e1y
    m5 = h2x * e2y * h1y - h2y * h2x * e1y
    m6 = h2y * h2x * e1y - e2y * h2y * h1x
    m7 = h2x * h2x * e1y - e2y * h2x * h1x
    det = h1x * m1 - h1y * m2
    Z = [(e1x * m1 - h1y * m3) / det, (h1x * m3 - e1x * m2) / det,
         (h1x * m4 - h1y * m5) / det, (h1x * m6 - h1y * m7) / det]
    rho = [np.abs(z) ** 2 / (mu * omega) for z in Z]
    phase = [np.mod(np.degrees(np.arctan(-z.imag / z.real)), 360.0) for z in Z]
    c = h1x * h2y
    ty = (h2z / h2y - (h1z * h2x) / c) / (1.0 - (h1y * h2x) / c)
    tx = (h1z - ty * h1y) / h1x
    return rho, phase, [tx, ty], Z


def write_results(stem, datasets):
    """{stem}.h5 with petgem's group/dataset paths (postprocessing.py:341-461):
    through h5py when it is installed, else with petgem_gb300.hdf5 (the same
    classic HDF5 format, no HDF5 library needed)."""
    path = stem + ".h5"
    try:
        import h5py
    except ImportError:
        from . import hdf5
        return hdf5.write(path, datasets)
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
