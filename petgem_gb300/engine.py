"""Device-resident forward-modelling engine (one GPU).

``DeviceMesh`` holds a tetrahedral mesh on the GPU together with everything
derived from it once per mesh (topology, DOF numbering, orientation tuples and
their moment tables, the CSR pattern and the PEC DOF list).  Per model
(conductivity, frequency, source) it assembles A and b, solves, and
interpolates the receivers.  Every computation runs in libpetgem_gb300.so;
torch only provides device memory and the current stream.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib

MU0 = 4.0 * math.pi * 1e-7     # petgem/solver.py:174


def _p(t):
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ws(nbytes, dev):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=dev)


def ndof_elem(p):
    return p * (p + 2) * (p + 3) // 2


def source_field(src):
    """Dipole moment vector after azimuth/dip rotation (petgem/hvfem.py:2303-2344,
    solver.py:255-266): rot(azimuth) rot(dip) (I L e_x)."""
    a = math.radians(src["azimuth"])
    b = math.radians(src["dip"])
    IL = float(src["current"]) * float(src["length"])
    # M1 (x-y) @ M2 (x-z) @ e_x
    v = np.array([math.cos(a) * math.cos(b), math.sin(a) * math.cos(b), math.sin(b)])
    return v * IL


class SolveInfo:
    def __init__(self, iterations, restarts, relres, status, relres_per_rhs, seconds=None):
        self.iterations = iterations
        self.restarts = restarts
        self.relres = relres
        self.status = status
        self.relres_per_rhs = relres_per_rhs
        self.seconds = seconds

    def __repr__(self):
        return (f"SolveInfo(iterations={self.iterations}, restarts={self.restarts}, relres={self.relres:.3e}, "
                f"status={self.status})")


class DeviceMesh:
    """Mesh, topology, DOF map, orientation tables and CSR pattern on one GPU."""

    def __init__(self, nodes, elemsN, p, device="cuda:0", pattern=True):
        if not 1 <= p <= 6:
            raise ValueError("basis order must be 1..6 (petgem/common.py:210-216)")
        self.device = torch.device(device)
        self.p = int(p)
        dev = self.device
        self.nodes = torch.as_tensor(np.ascontiguousarray(nodes, dtype=np.float64), device=dev).contiguous()
        self.elemsN = torch.as_tensor(np.ascontiguousarray(elemsN), device=dev).to(torch.int32).contiguous()
        self.T = int(self.elemsN.shape[0])
        self.n_nodes = int(self.nodes.shape[0])
        self._topology()
        self._dofs_orientation()
        self._tables()
        self._boundary()
        self.rowptr = self.col = None
        if pattern:
            self._pattern()

    # ---------------------------------------------------------------- per-mesh setup
    def _topology(self):
        dev, T = self.device, self.T
        i32 = dict(dtype=torch.int32, device=dev)
        self.elemsE = torch.empty((T, 6), **i32)
        self.elemsF = torch.empty((T, 4), **i32)
        edgesNodes = torch.empty((6 * T, 2), **i32)
        facesN = torch.empty((4 * T, 3), **i32)
        facesE = torch.empty((4 * T, 3), **i32)
        face_nelem = torch.empty(4 * T, **i32)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        status = torch.zeros(1, **i32)
        ws = _ws(_lib.query("pg_topology_workspace_bytes", T), dev)
        _lib.call("pg_topology", _p(self.elemsN), T, self.n_nodes, _p(self.elemsE), _p(self.elemsF), _p(edgesNodes),
                  _p(facesN), _p(facesE), _p(face_nelem), _p(counts), _p(status), _p(ws), ws.numel(), _s())
        c = counts.cpu().tolist()
        if int(status.item()) != 0:
            raise _lib.PetgemError("pg_topology", int(status.item()), "node index out of range in elemsN")
        self.nE, self.nF = int(c[0]), int(c[1])
        self.edgesNodes = edgesNodes[:self.nE].contiguous()
        self.facesN = facesN[:self.nF].contiguous()
        self.facesE = facesE[:self.nF].contiguous()
        self.face_nelem = face_nelem[:self.nF].contiguous()

    def _dofs_orientation(self):
        dev, T, p = self.device, self.T, self.p
        self.nd = ndof_elem(p)
        self.dofs = torch.empty((T, self.nd), dtype=torch.int32, device=dev)
        _lib.call("pg_connectivity_dofs", _p(self.elemsE), _p(self.elemsF), T, self.nE, self.nF, p, _p(self.dofs), _s())
        self.N = self.nE * p + self.nF * p * (p - 1) + T * (p * (p - 1) * (p - 2) // 2)
        self.eo = torch.empty((T, 6), dtype=torch.int8, device=dev)
        self.fo = torch.empty((T, 4), dtype=torch.int8, device=dev)
        _lib.call("pg_element_orientation", _p(self.elemsN), _p(self.elemsE), _p(self.edgesNodes), _p(self.elemsF),
                  _p(self.facesE), T, _p(self.eo), _p(self.fo), _s())

    def _tables(self):
        dev, T = self.device, self.T
        self.tuple_of_elem = torch.empty(T, dtype=torch.int32, device=dev)
        codes = torch.empty(min(T, 64 * 1296), dtype=torch.int32, device=dev)
        n = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_tuples_workspace_bytes", T), dev)
        _lib.call("pg_orientation_tuples", _p(self.eo), _p(self.fo), T, _p(self.tuple_of_elem), _p(codes), _p(n),
                  _p(ws), ws.numel(), _s())
        U = int(n.item())
        self.codes = codes[:U].contiguous()
        per = _lib.query("pg_table_doubles", self.p)
        self.tables = torch.empty(U * per, dtype=torch.float64, device=dev)
        _lib.call("pg_tuple_tables", _p(self.codes), U, self.p, _p(self.tables), _s())
        self.n_tuples = U

    def _boundary(self):
        dev, p = self.device, self.p
        cap = self.nE * p + self.nF * p * (p - 1)
        bnd = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
        nb = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_boundary_workspace_bytes", self.nE, self.nF), dev)
        _lib.call("pg_boundary_dofs", _p(self.face_nelem), _p(self.facesE), self.nE, self.nF, p, _p(bnd), _p(nb),
                  _p(ws), ws.numel(), _s())
        self.bnd = bnd[:int(nb.item())].contiguous()
        self.pec_flags = torch.empty(self.N, dtype=torch.uint8, device=dev)

    def _pattern(self):
        dev, T, p = self.device, self.T, self.p
        nl = _lib.query("pg_pattern_local_entities", p)
        M = T * nl * nl
        self.members = torch.empty(M, dtype=torch.int32, device=dev)
        pair_start = torch.empty(M + 1, dtype=torch.int32, device=dev)
        pair_colstart = torch.empty(M, dtype=torch.int32, device=dev)
        self.rowptr = torch.empty(self.N + 1, dtype=torch.int64, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_pattern_workspace_bytes", T, self.nE, self.nF, p), dev)
        _lib.call("pg_pattern_build", _p(self.elemsE), _p(self.elemsF), T, self.nE, self.nF, p, _p(self.members),
                  _p(pair_start), _p(pair_colstart), _p(self.rowptr), _p(counts), _p(ws), ws.numel(), _s())
        del ws
        c = counts.cpu().tolist()
        self.n_pairs, self.nnz = int(c[0]), int(c[1])
        self.pair_start = pair_start[:self.n_pairs + 1].contiguous()
        self.pair_colstart = pair_colstart[:self.n_pairs].contiguous()
        del pair_start, pair_colstart
        self.col = torch.empty(self.nnz, dtype=torch.int32, device=dev)
        _lib.call("pg_pattern_columns", _p(self.members), _p(self.pair_start), _p(self.pair_colstart), self.n_pairs,
                  _p(self.elemsE), _p(self.elemsF), T, self.nE, self.nF, p, _p(self.rowptr), _p(self.col), _s())
        # symmetric work list for the fused assembly
        self.pair_partner = torch.empty(self.n_pairs, dtype=torch.int32, device=dev)
        items = torch.empty(self.nnz, dtype=torch.int64, device=dev)
        nit = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_pattern_items_workspace_bytes", self.n_pairs, self.nnz), dev)
        _lib.call("pg_pattern_items", _p(self.members), _p(self.pair_start), self.n_pairs, _p(self.elemsE),
                  _p(self.elemsF), T, self.nE, self.nF, p, self.nnz, _p(self.pair_partner), _p(items), _p(nit),
                  _p(ws), ws.numel(), _s())
        self.n_items = int(nit.item())
        self.items = items[:self.n_items].contiguous()
        del items, ws

    # ---------------------------------------------------------------- per-model work
    def sigma_tensor(self, sigma):
        s = torch.as_tensor(np.ascontiguousarray(sigma, dtype=np.float64), device=self.device)
        if s.ndim == 1:
            s = torch.stack([s, s], dim=1)
        return s.contiguous()

    def elemental_matrices(self, sigma):
        """Batched elemental (M, K) f64 [T, nd, nd] (petgem/hvfem.py:223)."""
        s = self.sigma_tensor(sigma) if not torch.is_tensor(sigma) else sigma
        M = torch.empty((self.T, self.nd, self.nd), dtype=torch.float64, device=self.device)
        K = torch.empty_like(M)
        st = torch.zeros(1, dtype=torch.int32, device=self.device)
        _lib.call("pg_elemental_matrices", _p(self.nodes), _p(self.elemsN), _p(s), _p(self.tuple_of_elem),
                  _p(self.tables), self.T, self.p, _p(M), _p(K), _p(st), _s())
        if int(st.item()) != 0:
            raise _lib.PetgemError("pg_elemental_matrices", int(st.item()), "degenerate element")
        return M, K

    def element_coefficients(self, sigma, frequency, out=None, check=True, arithmetic="fp64"):
        """Per-element geometry coefficients [T, 12] (float64), or with
        arithmetic="df64" their (hi, lo) float32 pairs [T, 12, 2]."""
        s = self.sigma_tensor(sigma) if not torch.is_tensor(sigma) else sigma
        omu = 2.0 * math.pi * float(frequency) * MU0
        st = torch.zeros(1, dtype=torch.int32, device=self.device)
        if arithmetic == "df64":
            coef = out if out is not None else torch.empty((self.T, 12, 2), dtype=torch.float32, device=self.device)
            fn = "pg_element_coefficients_df"
        else:
            coef = out if out is not None else torch.empty((self.T, 12), dtype=torch.float64, device=self.device)
            fn = "pg_element_coefficients"
        _lib.call(fn, _p(self.nodes), _p(self.elemsN), _p(s), self.T, omu, _p(coef), _p(st), _s())
        if check and int(st.item()) != 0:
            raise _lib.PetgemError("pg_element_coefficients", int(st.item()), "degenerate element")
        return coef

    def tables_entry_major(self, arithmetic="fp64"):
        """Moment tables entry-major [U][NT][12] (float64, or (hi, lo) float32
        pairs for arithmetic="df64"), once per mesh."""
        key = "_tables_em_" + arithmetic
        if getattr(self, key, None) is None:
            n = self.tables.numel()
            t = torch.empty(n if arithmetic == "fp64" else 2 * n,
                            dtype=torch.float64 if arithmetic == "fp64" else torch.float32, device=self.device)
            _lib.call("pg_tuple_tables_entry_major", _p(self.tables), self.n_tuples, self.p,
                      0 if arithmetic == "fp64" else 1, _p(t), _s())
            setattr(self, key, t)
        return getattr(self, key)

    def tables_df(self):
        """Moment tables as (hi, lo) float32 pairs, table-major like self.tables (once per mesh)."""
        if getattr(self, "_tables_df", None) is None:
            t = torch.empty(2 * self.tables.numel(), dtype=torch.float32, device=self.device)
            _lib.call("pg_to_double_float", _p(self.tables), self.tables.numel(), _p(t), _s())
            self._tables_df = t
        return self._tables_df

    def pec_mask(self):
        """uint8 [N] flags of the PEC DOFs (once per mesh)."""
        if getattr(self, "_pec_mask", None) is None:
            f = torch.empty(self.N, dtype=torch.uint8, device=self.device)
            _lib.call("pg_pec_flags", _p(self.bnd), self.bnd.numel(), self.N, _p(f), _s())
            self._pec_mask = f
        return self._pec_mask

    def gradient_map(self, pec=True, vector=None):
        """The mesh's auxiliary map (pg_gradient_map; built once per variant,
        p <= 3): the discrete gradient G of the order-p H1 space and, with
        vector (default: p >= 2), the vector P1 fields after it; the
        correction of ``solve(precond="grad")`` applies a Jacobi step on every
        column.  pec=True drops the columns that touch a PEC DOF (CSEM
        systems, PEC applied); pec=False keeps every column (MT systems, whose
        boundary DOFs stay unknowns)."""
        vec = (self.p >= 2) if vector is None else bool(vector)
        cache = self.__dict__.setdefault("_grad", {})
        key = (bool(pec), vec)
        if key not in cache:
            dev = self.device
            nc, me = ctypes.c_int64(), ctypes.c_int64()
            _lib.call("pg_gradient_map_sizes", self.n_nodes, self.nE, self.nF, self.T, self.p, int(vec),
                      ctypes.byref(nc), ctypes.byref(me))
            nc, me = int(nc.value), int(me.value)
            g = GradientMap(nc, torch.empty(self.N + 1, dtype=torch.int64, device=dev),
                            torch.empty(me, dtype=torch.int32, device=dev),
                            torch.empty(me, dtype=torch.float64, device=dev),
                            torch.empty(nc + 1, dtype=torch.int64, device=dev),
                            torch.empty(me, dtype=torch.int32, device=dev),
                            torch.empty(me, dtype=torch.float64, device=dev))
            ws = _ws(_lib.query("pg_gradient_map_workspace_bytes", self.n_nodes, self.nE, self.nF, self.T,
                                self.n_tuples, self.p, int(vec)), dev)
            _lib.call("pg_gradient_map", _p(self.nodes), _p(self.elemsN), _p(self.elemsE), _p(self.elemsF),
                      _p(self.dofs), _p(self.tuple_of_elem), _p(self.codes), self.n_tuples, self.T, self.n_nodes,
                      self.nE, self.nF, self.p, int(vec), _p(self.pec_mask()) if pec else None, _p(g.rowptr),
                      _p(g.col), _p(g.val), _p(g.t_rowptr), _p(g.t_row), _p(g.t_val), _p(ws), ws.numel(), _s())
            cache[key] = g
        return cache[key]

    def records(self):
        """Assembly records (once per mesh): output / transpose position,
        first member and PEC flags of every item of the work list."""
        if getattr(self, "_records", None) is None:
            if self.col is None:
                self._pattern()
            rb = _lib.query("pg_assembly_record_bytes", self.nnz)
            r = torch.empty(self.n_items * rb, dtype=torch.uint8, device=self.device)
            st = torch.zeros(1, dtype=torch.int32, device=self.device)
            _lib.call("pg_assembly_records", _p(self.members), _p(self.pair_start), _p(self.pair_colstart),
                      _p(self.pair_partner), _p(self.items), self.n_items, _p(self.elemsE), _p(self.elemsF), self.T,
                      self.nE, self.nF, self.p, _p(self.rowptr), self.nnz, _p(self.pec_mask()), _p(r), _p(st), _s())
            if int(st.item()) != 0:
                raise _lib.PetgemError("pg_assembly_records", int(st.item()), "a CSR pair has more than 255 members")
            self._records = r
        return self._records

    def assemble(self, sigma, frequency, fused=True, out=None, coef=None, arithmetic="fp64", pec=False,
                 records=True):
        """A values (complex128 [nnz]): sum_e K_e - i omega mu M_e.

        arithmetic="fp64" multiplies the tables in FP64; "df64" in double-float
        (FP32 pairs, ~2^-48 relative rounding per product, FP64-class result).
        pec=True applies zeroRowsColumns(boundaries, diag=1) in the same pass
        (the matrix half of apply_pec; b still needs pec_rhs).
        coef: precomputed element_coefficients(..., arithmetic=arithmetic).
        records=True uses the per-mesh assembly records (pg_assemble_records),
        False the item list directly (pg_assemble_fused_ex); same values."""
        if self.col is None:
            self._pattern()
        vals = out if out is not None else torch.empty(self.nnz, dtype=torch.complex128, device=self.device)
        if arithmetic not in ("fp64", "df64"):
            raise ValueError(f"arithmetic={arithmetic!r}: fp64 or df64")
        if not fused and (arithmetic != "fp64" or pec):
            raise ValueError("arithmetic='df64' and pec=True need the fused assembly")
        if fused:
            if coef is None:
                coef = self.element_coefficients(sigma, frequency, arithmetic=arithmetic)
            want = torch.float64 if arithmetic == "fp64" else torch.float32
            if coef.dtype != want or coef.numel() != self.T * 12 * (1 if arithmetic == "fp64" else 2):
                raise ValueError("coef does not match the arithmetic")
            mode = 0 if arithmetic == "fp64" else 1
            if records:
                _lib.call("pg_assemble_records", _p(coef), _p(self.tuple_of_elem), _p(self.tables_entry_major(arithmetic)),
                          _p(self.members), _p(self.records()), self.n_items, self.nnz, self.p, mode, int(pec),
                          _p(vals), _s())
            else:
                tb = self.tables if mode == 0 else self.tables_df()
                _lib.call("pg_assemble_fused_ex", _p(coef), _p(self.tuple_of_elem), _p(tb), _p(self.members),
                          _p(self.pair_start), _p(self.pair_colstart), _p(self.pair_partner), _p(self.items),
                          self.n_items, self.n_pairs, _p(self.elemsE), _p(self.elemsF), self.T, self.nE, self.nF,
                          self.p, _p(self.rowptr), _p(self.pec_mask() if pec else None), mode, _p(vals), _s())
        else:
            M, K = self.elemental_matrices(sigma)
            omu = 2.0 * math.pi * float(frequency) * MU0
            _lib.call("pg_assemble_values", _p(M), _p(K), _p(self.members), _p(self.pair_start),
                      _p(self.pair_colstart), self.n_pairs, _p(self.elemsE), _p(self.elemsF), self.T, self.nE, self.nF,
                      self.p, _p(self.rowptr), omu, _p(vals), _s())
        return vals

    def pec_rhs(self, b):
        """b[boundaries] = 0 for every column of b (solver.py:565-567)."""
        nrhs = 1 if b.ndim == 1 else int(b.shape[1])
        _lib.call("pg_pec_rhs", _p(self.bnd), self.bnd.numel(), nrhs, _p(b), _s())
        return b

    def locate(self, pts, tol=1e-12):
        pts_t = torch.as_tensor(np.ascontiguousarray(np.atleast_2d(pts), dtype=np.float64), device=self.device)
        out = torch.empty(pts_t.shape[0], dtype=torch.int32, device=self.device)
        _lib.call("pg_locate_points", _p(self.nodes), _p(self.elemsN), self.T, _p(pts_t), pts_t.shape[0], tol,
                  _p(out), _s())
        return pts_t, out

    def locate_source(self, src):
        """Element containing the source point (petgem/preprocessing.py:414-425), device int32 [1]."""
        _, elem = self.locate(np.asarray(src["position"], dtype=np.float64))
        return elem

    def source_rhs(self, src, elem, b, status=None):
        """b += i omega mu (field . N_e(position)) on the device (no host sync)."""
        pos = np.asarray(src["position"], dtype=np.float64)
        field = source_field(src)
        omu = 2.0 * math.pi * float(src["frequency"]) * MU0
        st = status if status is not None else torch.zeros(1, dtype=torch.int32, device=self.device)
        pos_c = (ctypes.c_double * 3)(*pos.tolist())
        fld_c = (ctypes.c_double * 3)(*field.tolist())
        _lib.call("pg_source_rhs", _p(self.nodes), _p(self.elemsN), _p(self.eo), _p(self.fo), _p(self.dofs), self.p,
                  _p(elem), ctypes.cast(pos_c, ctypes.c_void_p), ctypes.cast(fld_c, ctypes.c_void_p), 0.0, omu,
                  _p(b), _p(st), _s())
        return st

    def source_vector(self, src, b=None):
        """Point-dipole RHS (petgem/solver.py:247-316); returns (b, source element)."""
        if b is None:
            b = torch.zeros(self.N, dtype=torch.complex128, device=self.device)
        elem = self.locate_source(src)
        st = self.source_rhs(src, elem, b)
        s = int(st.item())
        if s != 0:
            raise _lib.PetgemError("pg_source_rhs", s, "source not located in the computational domain")
        return b, int(elem.item())

    def apply_pec(self, vals, b=None):
        """zeroRowsColumns(boundaries, diag=1) and b[boundaries] = 0 (solver.py:552-577)."""
        _lib.call("pg_apply_pec", _p(self.rowptr), _p(self.col), _p(vals), self.N, _p(self.bnd), self.bnd.numel(),
                  _p(b), _p(self.pec_flags), _s())
        return vals, b

    def solve(self, vals, b, x0=None, rtol=1e-8, restart=30, max_it=20000, precision="fp64", reorth=False,
              raise_on_fail=True, ksp="gmres", check_every=50, precond="block", inner_rtol=None, pec=True):
        """Solve A x = b for this mesh's CSR pattern (see solve_csr).
        precond="block": entity block-Jacobi (each edge / face / volume's
        diagonal block factored L D L^T; COCG and GMRES); "jacobi": diagonal;
        "grad": diagonal Jacobi plus the auxiliary-space correction
        D^-1 + G diag(G^T A G)^-1 G^T, G = gradient_map() (the discrete
        gradients and, for p >= 2, the vector P1 fields; COCG in fp64, df64 or
        ir32, GMRES in fp64 or mixed;
        p <= 3; gradient_map; pec=False for systems without PEC rows, e.g.
        MT, which want fp64: their true residual has an FP64 floor)."""
        if precond not in ("block", "jacobi", "grad"):
            raise ValueError(f"unknown preconditioner {precond!r} (block, jacobi, grad)")
        if precond == "grad" and not pec and precision != "fp64":
            # without PEC rows the air's gradient components make the true
            # residual noisy at the FP64 floor; only the FP64 recurrence, which
            # never restarts from it, stays stable there
            raise ValueError("precond='grad' with pec=False (MT systems) runs in precision='fp64'")
        blocks = (self.p, self.nE, self.nF, self.T) if precond == "block" else None
        gradient = self.gradient_map(pec) if precond == "grad" else None
        return solve_csr(self.rowptr, self.col, vals, b, x0=x0, rtol=rtol, restart=restart, max_it=max_it,
                         precision=precision, reorth=reorth, raise_on_fail=raise_on_fail, ksp=ksp,
                         check_every=check_every, blocks=blocks, inner_rtol=inner_rtol, gradient=gradient)

    def solve_frequencies(self, vals0, frequency0, b, frequencies, precond="jacobi", **kw):
        """Columns of b (complex128 [N, k]) at their own frequencies in one
        solve: vals0 is A assembled (PEC applied) at frequency0; see
        solve_csr_frequencies.  precond="grad" adds the gradient correction."""
        scale = [float(f) / float(frequency0) for f in frequencies]
        gradient = self.gradient_map() if precond == "grad" else None
        return solve_csr_frequencies(self.rowptr, self.col, vals0, b, scale, gradient=gradient, **kw)

    def receiver_fields(self, x, receivers, frequency):
        """(fields complex128 [R', 6], kept mask) like petgem fieldInterpolator
        (postprocessing.py:479-616): receivers outside the mesh are dropped."""
        pts_t, elem = self.locate(receivers)
        R = pts_t.shape[0]
        F = torch.empty((R, 6), dtype=torch.complex128, device=self.device)
        omu = 2.0 * math.pi * float(frequency) * MU0
        _lib.call("pg_gather_fields", _p(x.contiguous()), _p(self.nodes), _p(self.elemsN), _p(self.eo), _p(self.fo),
                  _p(self.dofs), self.p, _p(pts_t), _p(elem), R, omu, _p(F), _s())
        keep = (elem >= 0)
        return F[keep], keep

    # ---------------------------------------------------------------- MT excitation
    def mt_boundary(self):
        """Boundary faces, their elements / local faces / box sides and the
        per-DOF scatter plan of the MT right-hand side (once per mesh)."""
        if getattr(self, "_mt", None) is not None:
            return self._mt
        dev, nF = self.device, self.nF
        bface = torch.empty(nF, dtype=torch.int32, device=dev)
        belem = torch.empty(nF, dtype=torch.int32, device=dev)
        blocal = torch.empty(nF, dtype=torch.int8, device=dev)
        nb = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_boundary_faces_workspace_bytes", nF), dev)
        _lib.call("pg_boundary_faces", _p(self.elemsF), _p(self.face_nelem), self.T, nF, _p(bface), _p(belem),
                  _p(blocal), _p(nb), _p(ws), ws.numel(), _s())
        n = int(nb.item())
        bface, belem, blocal = bface[:n].contiguous(), belem[:n].contiguous(), blocal[:n].contiguous()
        lo = torch.amin(self.nodes, dim=0).cpu().numpy()
        hi = torch.amax(self.nodes, dim=0).cpu().numpy()
        bbox = np.array([lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]], dtype=np.float64)
        plane = torch.empty(n, dtype=torch.int8, device=dev)
        cz = torch.empty(n, dtype=torch.float64, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("pg_face_planes", _p(self.nodes), _p(self.elemsN), _p(self.facesN), _p(bface), _p(belem),
                  _p(blocal), n, ctypes.c_void_p(bbox.ctypes.data), _p(plane), _p(cz), _p(st), _s())
        if int(st.item()) != 0:
            raise _lib.PetgemError("pg_face_planes", int(st.item()),
                                   "a boundary face lies on no side of the bounding box (MT needs a box domain)")
        m = n * self.nd
        order = torch.empty(m, dtype=torch.int32, device=dev)
        seg_start = torch.empty(m + 1, dtype=torch.int32, device=dev)
        seg_dof = torch.empty(m, dtype=torch.int32, device=dev)
        nseg = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(_lib.query("pg_mt_plan_workspace_bytes", n, self.p), dev)
        _lib.call("pg_mt_plan", _p(self.dofs), _p(belem), n, self.p, self.N, _p(order), _p(seg_start), _p(seg_dof),
                  _p(nseg), _p(ws), ws.numel(), _s())
        self._mt = {"bface": bface, "belem": belem, "blocal": blocal, "plane": plane, "centroid_z": cz,
                    "bbox": bbox, "order": order, "seg_start": seg_start, "seg_dof": seg_dof,
                    "n_seg": int(nseg.item()), "n": n}
        return self._mt

    def mt_face_z(self, rule):
        """z of every (boundary face, rule point): f64 [n_bfaces, n_rule] on the device.
        rule: (points (n, 2), weights (n,)) on the triangle (0,0),(1,0),(0,1)."""
        bd = self.mt_boundary()
        r = self._rule_tensor(rule)
        z = torch.empty((bd["n"], r.shape[0]), dtype=torch.float64, device=self.device)
        _lib.call("pg_mt_face_z", _p(self.nodes), _p(self.elemsN), _p(bd["belem"]), _p(bd["blocal"]), bd["n"],
                  _p(r), r.shape[0], _p(z), _s())
        return z

    def _rule_tensor(self, rule):
        pts, w = rule
        r = np.concatenate([np.asarray(pts, dtype=np.float64).reshape(-1, 2),
                            np.asarray(w, dtype=np.float64).reshape(-1, 1)], axis=1)
        return torch.as_tensor(np.ascontiguousarray(r), device=self.device)

    def mt_field(self, sigma, frequency, rule, n_nodes=10 ** 6):
        """u at every boundary-face rule point (complex [n_bfaces, n_rule]): the
        1-D MT field of the right-side (x = max) boundary profile
        (petgem/solver.py:318-395, mt1d.eval_MT1D on the host)."""
        from . import mt1d
        bd = self.mt_boundary()
        z = self.mt_face_z(rule).cpu().numpy()
        right = (bd["plane"] == 3)
        cz = bd["centroid_z"][right].cpu().numpy()
        s = self.sigma_tensor(sigma) if not torch.is_tensor(sigma) else sigma
        s4 = s[bd["belem"].long()[right], 0].cpu().numpy()
        omega = 2.0 * math.pi * float(frequency)
        u = mt1d.eval_MT1D(bd["bbox"][5], bd["bbox"][4], 1.0, 0.0, s4, cz, omega, MU0, int(n_nodes), 1, z)
        return torch.as_tensor(np.ascontiguousarray(u, dtype=np.complex128), device=self.device)

    def mt_rhs(self, sigma, frequency, polarizations=("x", "y"), rule=None, u=None, n_nodes=10 ** 6):
        """MT plane-wave right-hand sides b complex128 [N, npol] (one column per
        polarisation, RHS fastest, ready for a batched solve), petgem's
        solver.py:318-512.  rule defaults to a triangle rule exact to degree
        2p + 2; u (the 1-D field at the rule points) is computed when None."""
        from . import mt1d
        bd = self.mt_boundary()
        rule = rule if rule is not None else mt1d.triangle_rule(2 * self.p + 2)
        if u is None:
            u = self.mt_field(sigma, frequency, rule, n_nodes)
        u = u.to(torch.complex128).contiguous()
        r = self._rule_tensor(rule)
        pols = [{"x": 1, "y": 2}[str(q)] for q in polarizations]
        b = torch.zeros((self.N, len(pols)), dtype=torch.complex128, device=self.device)
        omu = 2.0 * math.pi * float(frequency) * MU0
        ws = _ws(_lib.query("pg_mt_rhs_workspace_bytes", bd["n"], self.p), self.device)
        for k, pol in enumerate(pols):
            _lib.call("pg_mt_rhs", _p(self.nodes), _p(self.elemsN), _p(self.eo), _p(self.fo), self.p, _p(bd["belem"]),
                      _p(bd["blocal"]), _p(bd["plane"]), bd["n"], _p(r), r.shape[0], _p(u), pol, 0.0, omu,
                      _p(bd["order"]), _p(bd["seg_start"]), _p(bd["seg_dof"]), bd["n_seg"], _p(b), len(pols), k,
                      _p(ws), ws.numel(), _s())
        return b

    def node_fields(self, x, frequency):
        """Nodal E and H (complex128 [n_nodes, 6]) for visualisation
        (petgem/postprocessing.py:173-260)."""
        out = torch.empty((self.n_nodes, 6), dtype=torch.complex128, device=self.device)
        ws = _ws(_lib.query("pg_node_fields_workspace_bytes", self.T, self.n_nodes), self.device)
        omu = 2.0 * math.pi * float(frequency) * MU0
        _lib.call("pg_node_fields", _p(x.contiguous()), _p(self.nodes), _p(self.elemsN), _p(self.eo), _p(self.fo),
                  _p(self.dofs), self.p, self.T, self.n_nodes, omu, _p(out), _p(ws), ws.numel(), _s())
        return out

    def receiver_adjoint(self, weights, receivers, b=None):
        """b += G^T w: the transpose of the E part of receiver_fields, with
        weights complex128 [R, 3] per (kept or dropped) receiver in the order
        given; receivers outside the mesh contribute nothing."""
        pts_t, elem = self.locate(receivers)
        R = pts_t.shape[0]
        w = weights.to(torch.complex128).contiguous()
        if w.shape != (R, 3):
            raise ValueError(f"weights must be [{R}, 3]")
        if b is None:
            b = torch.zeros(self.N, dtype=torch.complex128, device=self.device)
        ws = _ws(_lib.query("pg_receiver_adjoint_workspace_bytes", self.p, R), self.device)
        _lib.call("pg_receiver_adjoint", _p(self.nodes), _p(self.elemsN), _p(self.eo), _p(self.fo), _p(self.dofs),
                  self.p, _p(pts_t), _p(elem), R, _p(w), _p(b), _p(ws), ws.numel(), _s())
        return b

    def element_mass_bilinear(self, coef, x, y):
        """out[e] = y_e^T (-omega mu M_e) x_e (complex128 [T]); coef from
        element_coefficients (FP64) at the frequency of interest."""
        out = torch.empty(self.T, dtype=torch.complex128, device=self.device)
        _lib.call("pg_element_mass_bilinear", _p(coef), _p(self.tuple_of_elem), _p(self.tables), _p(self.dofs),
                  _p(x.contiguous()), _p(y.contiguous()), self.T, self.p, _p(out), _s())
        return out

    def spmv(self, vals, x):
        y = torch.empty_like(x)
        nrhs = 1 if x.ndim == 1 else int(x.shape[1])
        _lib.call("pg_spmv_z", _p(self.rowptr), _p(self.col), _p(vals), self.N, _p(x.contiguous()), _p(y), nrhs, _s())
        return y


class GradientMap:
    """Discrete gradient G (CSR, real, rows = H(curl) DOFs, n_cols H1
    columns) and its transpose, as pg_gradient_map writes them."""

    def __init__(self, n_cols, rowptr, col, val, t_rowptr, t_row, t_val):
        self.n_cols = n_cols
        self.rowptr, self.col, self.val = rowptr, col, val
        self.t_rowptr, self.t_row, self.t_val = t_rowptr, t_row, t_val

    @property
    def nnz(self):
        return int(self.rowptr[-1].item())


def _n_rows(rowptr):
    return int(rowptr.numel()) - 1


def _set_gradient(o, g):
    """Point solver options (pg_cocg_opts / pg_gmres_opts) at a GradientMap."""
    o.grad_cols = g.n_cols
    o.grad_rowptr, o.grad_col, o.grad_val = _p(g.rowptr), _p(g.col), _p(g.val)
    o.gradt_rowptr, o.gradt_row, o.gradt_val = _p(g.t_rowptr), _p(g.t_row), _p(g.t_val)


def _check_csr(name, rowptr, col, vals, b):
    """CSR system on the GPU: rowptr int64 [N+1], col int32 [nnz], vals
    complex128 [nnz], b complex128 [N] or [N, k]; raises ValueError before
    anything reaches the library."""
    if rowptr.dtype != torch.int64 or col.dtype != torch.int32:
        raise ValueError(f"{name}: rowptr must be int64 and col int32 (got {rowptr.dtype}, {col.dtype})")
    if vals.dtype != torch.complex128 or b.dtype != torch.complex128:
        raise ValueError(f"{name}: vals and b must be complex128 (got {vals.dtype}, {b.dtype})")
    if rowptr.ndim != 1 or col.ndim != 1 or vals.ndim != 1 or b.ndim not in (1, 2):
        raise ValueError(f"{name}: rowptr, col, vals must be 1-D and b [N] or [N, k]")
    if col.numel() != vals.numel() or b.shape[0] != rowptr.numel() - 1:
        raise ValueError(f"{name}: sizes disagree (rows {rowptr.numel() - 1}, b {tuple(b.shape)}, "
                         f"col {col.numel()}, vals {vals.numel()})")
    # the library reads rowptr, col and vals through their data pointers
    for nm, t in (("rowptr", rowptr), ("col", col), ("vals", vals)):
        if not t.is_contiguous():
            raise ValueError(f"{name}: {nm} must be contiguous")
    devs = {t.device for t in (rowptr, col, vals, b)}
    if len(devs) != 1 or next(iter(devs)).type != "cuda":
        raise ValueError(f"{name}: every array must be on the same CUDA device (got {sorted(map(str, devs))})")


def _new_x(name, b, x0):
    """The solution buffer: row-major [N] or [N, k] like b (the kernels write
    x through its data pointer), zero or a contiguous copy of x0."""
    if x0 is None:
        return torch.zeros(tuple(b.shape), dtype=b.dtype, device=b.device)
    if tuple(x0.shape) != tuple(b.shape) or x0.dtype != b.dtype or x0.device != b.device:
        raise ValueError(f"{name}: x0 must match b (shape {tuple(b.shape)}, {b.dtype}, {b.device}); got "
                         f"{tuple(x0.shape)}, {x0.dtype}, {x0.device}")
    return x0.contiguous().clone()


def solve_csr(rowptr, col, vals, b, x0=None, rtol=1e-8, restart=30, max_it=20000, precision="fp64", reorth=False,
              raise_on_fail=True, ksp="gmres", check_every=50, blocks=None, inner_rtol=None, gradient=None):
    """Solve A x = b for a CSR matrix on the GPU (rowptr int64 [N+1], col
    int32 [nnz], vals complex128 [nnz]); b complex128 [N] or [N, k]
    (k in 1,2,4,8,16,32).  The KSPSolve of petgem/solver.py:584-594.

    ksp="gmres": right-preconditioned restarted GMRES(restart) (PETSc -ksp_type gmres,
                 -pc_type jacobi, or bjacobi with blocks);
    ksp="cocg":  Jacobi-scaled COCG for complex-symmetric A.
    precision="fp64" (complex128), "mixed" (complex64 matrix/SpMV, FP64 recurrence and
    refinement), "df64" (COCG only: double-float arithmetic on the FP32 pipes, FP64-class accuracy)
    or "ir32" (COCG only: FP64 iterative refinement of the true residual around complex64 inner
    solves, each restarted from the FP64 residual and run until its residual has dropped by
    inner_rtol, default 1e-2, or 1e-4 with the gradient correction; max_it counts inner iterations,
    info.restarts the refinement steps).
    Convergence: true residual ||b - A x|| <= rtol ||b|| in FP64.
    blocks=(p, n_edges, n_faces, n_elements): entity block-Jacobi on a pattern
    built by DeviceMesh (rows of one entity share their columns): COCG runs on
    S A S^T (S = D^-1/2 L^-1 per block), GMRES on A M^-1 (M^-1 = A_aa^-1 per
    block, right preconditioning: PETSc -pc_type bjacobi with one block per
    edge / face / element).
    gradient: a GradientMap (DeviceMesh.gradient_map) for the auxiliary-space
    correction: the preconditioner D^-1 + G diag(G^T A G)^-1 G^T, G the map
    with or without its vector P1 columns (diagonal Jacobi; COCG in fp64,
    df64 or ir32, GMRES in fp64 or mixed on the right).
    """
    _check_csr(f"solve_csr({ksp})", rowptr, col, vals, b)
    if gradient is not None:
        if blocks is not None:
            raise ValueError("the gradient correction is implemented with diagonal Jacobi (blocks=None)")
        if int(gradient.rowptr.numel()) != _n_rows(rowptr) + 1:
            raise ValueError("solve_csr: the gradient map's rows do not match the matrix")
    N = int(rowptr.numel()) - 1
    nnz = int(col.numel())
    nrhs = 1 if b.ndim == 1 else int(b.shape[1])
    x = _new_x(f"solve_csr({ksp})", b, x0)
    prec = {"fp64": 0, "mixed": 1, "df64": 2, "ir32": 3}[precision]
    if prec >= 2 and ksp != "cocg":
        raise ValueError(f"precision={precision!r} is implemented for ksp='cocg'")
    res = _lib.GmresResult()
    rr = (ctypes.c_double * nrhs)()
    lib = _lib.load()
    if ksp == "gmres":
        o = _lib.GmresOpts()
        lib.pg_gmres_default_opts(ctypes.byref(o))
        o.restart, o.max_it, o.rtol, o.precision, o.reorth = int(restart), int(max_it), float(rtol), prec, int(reorth)
        if blocks is not None:
            o.block_p, o.block_edges, o.block_faces, o.block_volumes = (int(v) for v in blocks)
        if gradient is not None:
            _set_gradient(o, gradient)
        nbytes = _lib.query("pg_gmres_workspace_bytes", N, nnz, nrhs, ctypes.byref(o))
        fn = lib.pg_gmres
    elif ksp == "cocg":
        o = _lib.CocgOpts()
        lib.pg_cocg_default_opts(ctypes.byref(o))
        o.max_it, o.rtol, o.precision, o.check_every = int(max_it), float(rtol), prec, int(check_every)
        if inner_rtol is not None:
            o.inner_rtol = float(inner_rtol)   # else the solver's default (1e-2; 1e-4 with gradient)
        if blocks is not None:
            o.block_p, o.block_edges, o.block_faces, o.block_volumes = (int(v) for v in blocks)
        if gradient is not None:
            _set_gradient(o, gradient)
        nbytes = _lib.query("pg_cocg_workspace_bytes", N, nnz, nrhs, ctypes.byref(o))
        fn = lib.pg_cocg
    else:
        raise ValueError(f"unknown ksp type {ksp!r} (gmres, cocg)")
    ws = _ws(nbytes + 256, b.device)
    st = fn(_p(rowptr), _p(col), _p(vals), N, nnz, _p(b.contiguous()), _p(x), nrhs,
            ctypes.byref(o), ctypes.byref(res), ctypes.cast(rr, ctypes.c_void_p), _p(ws), ws.numel(), _s())
    info = SolveInfo(int(res.iterations), int(res.restarts), float(res.relres), int(st), list(rr))
    if st != 0 and (raise_on_fail or st != -7):
        msg = lib.pg_last_error()
        raise _lib.PetgemError(f"pg_{ksp}", st, msg.decode() if msg else "")
    return x, info


def solve_csr_frequencies(rowptr, col, vals0, b, col_scale, x0=None, rtol=1e-8, max_it=100000, raise_on_fail=True,
                          check_every=50, gradient=None):
    """Several frequencies in one double-float COCG: column j of b (complex128
    [N, k], k in 1,2,4,8,16,32) is solved with (Re A0 + i s_j Im A0), where
    vals0 = A0 = K - i omega_0 mu M (PEC applied) and s_j = omega_j / omega_0.
    One matrix read per iteration serves every column.  gradient: a
    GradientMap for the gradient correction (see solve_csr)."""
    if b.ndim != 2:
        raise ValueError("b must be [N, k]")
    _check_csr("solve_csr_frequencies", rowptr, col, vals0, b)
    N = int(rowptr.numel()) - 1
    nnz = int(col.numel())
    k = int(b.shape[1])
    sc = np.ascontiguousarray(np.asarray(col_scale, dtype=np.float64).reshape(-1))
    if sc.size != k:
        raise ValueError("one frequency scale per column")
    x = _new_x("solve_csr_frequencies", b, x0)
    lib = _lib.load()
    o = _lib.CocgOpts()
    lib.pg_cocg_default_opts(ctypes.byref(o))
    o.max_it, o.rtol, o.precision, o.check_every = int(max_it), float(rtol), 2, int(check_every)
    if gradient is not None:
        _set_gradient(o, gradient)
    res = _lib.GmresResult()
    rr = (ctypes.c_double * k)()
    ws = _ws(_lib.query("pg_cocg_multifreq_workspace_bytes", N, nnz, k, ctypes.byref(o)) + 256, b.device)
    st = lib.pg_cocg_multifreq(_p(rowptr), _p(col), _p(vals0), N, nnz, _p(b.contiguous()), _p(x), k,
                               ctypes.c_void_p(sc.ctypes.data), ctypes.byref(o), ctypes.byref(res),
                               ctypes.cast(rr, ctypes.c_void_p), _p(ws), ws.numel(), _s())
    info = SolveInfo(int(res.iterations), int(res.restarts), float(res.relres), int(st), list(rr))
    if st != 0 and (raise_on_fail or st != -7):
        msg = lib.pg_last_error()
        raise _lib.PetgemError("pg_cocg_multifreq", st, msg.decode() if msg else "")
    return x, info


def concat_systems(systems):
    """Block-diagonal CSR of several systems [(rowptr, col, vals, b), ...]:
    (rowptr, col, vals, b, seg_rows) with system j in rows seg_rows[j] ..
    seg_rows[j+1]-1 and its columns shifted by seg_rows[j]."""
    rps, cols, vals, bs, rows, nz = [], [], [], [], [0], 0
    for rp, c, v, b in systems:
        n_j = int(rp.numel()) - 1
        rps.append(rp[:-1] + nz)
        cols.append(c + rows[-1])
        vals.append(v)
        bs.append(b)
        nz += int(c.numel())
        rows.append(rows[-1] + n_j)
    dev = systems[0][0].device
    rowptr = torch.cat(rps + [torch.tensor([nz], dtype=torch.int64, device=dev)])
    return (rowptr, torch.cat(cols).to(torch.int32), torch.cat(vals), torch.cat(bs),
            np.asarray(rows, dtype=np.int64))


def concat_gradients(gradients, rows):
    """Block-diagonal GradientMap of several systems' maps: system j's rows
    shifted by rows[j] and its columns by the columns before it."""
    rps, cols, vals, trps, trows, tvals = [], [], [], [], [], []
    nz, c0 = 0, 0
    for j, g in enumerate(gradients):
        n_j = int(g.rowptr.numel()) - 1
        if n_j != int(rows[j + 1] - rows[j]):
            raise ValueError(f"gradient map {j}: its rows do not match system {j}")
        e = g.nnz
        rps.append(g.rowptr[:-1] + nz)
        trps.append(g.t_rowptr[:-1] + nz)
        cols.append(g.col[:e] + c0)
        vals.append(g.val[:e])
        trows.append(g.t_row[:e] + int(rows[j]))
        tvals.append(g.t_val[:e])
        nz += e
        c0 += g.n_cols
    dev = gradients[0].rowptr.device
    end = torch.tensor([nz], dtype=torch.int64, device=dev)
    return GradientMap(c0, torch.cat(rps + [end]), torch.cat(cols).to(torch.int32), torch.cat(vals),
                       torch.cat(trps + [end]), torch.cat(trows).to(torch.int32), torch.cat(tvals))


def solve_csr_segments(systems, blocks=None, rtol=1e-8, max_it=100000, raise_on_fail=True, check_every=50,
                       gradients=None):
    """Several independent systems in one double-float COCG (pg_cocg_segments).

    systems: [(rowptr int64 [n_j+1], col int32, vals complex128, b complex128
    [n_j] or [n_j, k]), ...], every b with the same k (1,2,4,8,16,32).  Each
    system keeps its own scalars and convergence test (true residual <= rtol
    ||b_j|| per column); every kernel launch and graph replay serves all of
    them.  blocks: None (diagonal Jacobi) or (p, [(n_edges, n_faces,
    n_elements) per system]) for entity block-Jacobi.  gradients: None or
    one GradientMap per system (DeviceMesh.gradient_map) for the gradient
    correction (diagonal scaling).  Returns ([x_j], info) with
    info.relres_per_rhs and info.its_per_rhs per (system, rhs)."""
    if not systems:
        raise ValueError("no systems")
    for j, (rp, c, v, bj) in enumerate(systems):
        _check_csr(f"solve_csr_segments(system {j})", rp, c, v, bj)
    ks = {1 if b.ndim == 1 else int(b.shape[1]) for _, _, _, b in systems}
    if len(ks) != 1:
        raise ValueError("every system needs the same number of right-hand sides")
    k = ks.pop()
    rowptr, col, vals, b, rows = concat_systems(systems)
    if k > 1:
        b = b.reshape(-1, k)
    S = len(systems)
    N, nnz = int(rows[-1]), int(col.numel())
    lib = _lib.load()
    o = _lib.CocgOpts()
    lib.pg_cocg_default_opts(ctypes.byref(o))
    o.max_it, o.rtol, o.precision, o.check_every = int(max_it), float(rtol), 2, int(check_every)
    ents = None
    if blocks is not None:
        o.block_p = int(blocks[0])
        ents = np.ascontiguousarray(np.asarray(blocks[1], dtype=np.int64).reshape(S, 3))
    gmap = None
    if gradients is not None:
        if blocks is not None or len(gradients) != S:
            raise ValueError("gradients: one map per system, with diagonal scaling (blocks=None)")
        gmap = concat_gradients(gradients, rows)
        _set_gradient(o, gmap)
    ents_p = ctypes.c_void_p(ents.ctypes.data) if ents is not None else ctypes.c_void_p(0)
    rows_p = ctypes.c_void_p(rows.ctypes.data)
    nbytes = _lib.query("pg_cocg_segments_workspace_bytes", N, nnz, k, rows_p, S, ents_p, ctypes.byref(o))
    if nbytes == 0:
        raise ValueError("pg_cocg_segments: bad systems (empty, k not 1..32, or block counts not matching rows)")
    ws = _ws(nbytes + 256, b.device)
    x = _new_x("solve_csr_segments", b, None)
    res = _lib.GmresResult()
    rr = np.zeros(S * k, dtype=np.float64)
    its = np.zeros(S * k, dtype=np.int64)
    st = lib.pg_cocg_segments(_p(rowptr), _p(col), _p(vals), N, nnz, rows_p, S, ents_p, _p(b.contiguous()), _p(x), k,
                              ctypes.byref(o), ctypes.byref(res), ctypes.c_void_p(rr.ctypes.data),
                              ctypes.c_void_p(its.ctypes.data), _p(ws), ws.numel(), _s())
    info = SolveInfo(int(res.iterations), int(res.restarts), float(res.relres), int(st), rr.reshape(S, k).tolist())
    info.its_per_rhs = its.reshape(S, k).tolist()
    if st != 0 and (raise_on_fail or st != -7):
        msg = lib.pg_last_error()
        raise _lib.PetgemError("pg_cocg_segments", st, msg.decode() if msg else "")
    xs = [x[int(rows[j]):int(rows[j + 1])] for j in range(S)]
    return xs, info
