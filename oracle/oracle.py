"""ORACLE - test infrastructure only.

ctypes front end of oracle/_build/liboracle.so, the CPU restatement of the
PUNC++ particle path (see oracle.cpp for the parity status, which is
UNPINNED against the reference binary: the reference needs DOLFIN, PETSc and
Boost, none of which exist here).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module, as the checker.

The CircuitCM logic (punc/src/object_CM.cpp:53-376, punc/src/object.cpp:80-135)
is restated here in numpy because its matrices are 2n x 2n with n objects.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_SIG = {
    "or_create": ([_D, C.c_int64, _I64, C.c_int64, _I64, _I32, C.c_int64, _I64, C.c_int64, C.c_double, _I32], C.c_void_p),
    "or_free": ([C.c_void_p], None),
    "or_table_size": ([C.c_void_p, C.c_int32], C.c_int64),
    "or_table": ([C.c_void_p, C.c_int32, C.c_void_p], None),
    "or_locate": ([C.c_void_p, _D, C.c_int64, _I64], None),
    "or_add_particles": ([C.c_void_p, _D, _D, C.c_int64, C.c_double, C.c_double], C.c_int64),
    "or_num_particles": ([C.c_void_p], C.c_int64),
    "or_get_particles": ([C.c_void_p, _D, _D, _D, _D, _I64, _I64], None),
    "or_set_particles": ([C.c_void_p, _D, _D, _D, _D, _I64, _I64, C.c_int64], None),
    "or_efield_dg0": ([C.c_void_p, _D, _D, _D], None),
    "or_boris": ([C.c_void_p, _D, _D, C.c_double, C.c_int32], C.c_double),
    "or_accel": ([C.c_void_p, _D, C.c_double, C.c_int32], C.c_double),
    "or_esolver_rhs": ([C.c_void_p, _D, _D], None),
    "or_potential_energy": ([C.c_void_p, _D], C.c_double),
    "or_save_population": ([C.c_void_p, C.c_char_p, C.c_int32], C.c_int32),
    "or_density_cg1": ([C.c_void_p, C.c_double, C.c_double, _D, _D], None),
    "or_density_dg0": ([C.c_void_p, C.c_double, C.c_double, _D, _D], None),
    "or_statistics": ([C.c_void_p, _D], None),
    "or_accel_cg1": ([C.c_void_p, _D, C.c_double, C.c_int32], C.c_double),
    "or_boris_cg1": ([C.c_void_p, _D, _D, C.c_double, C.c_int32], C.c_double),
    "or_move": ([C.c_void_p, C.c_double, _D, C.c_int32], None),
    "or_update": ([C.c_void_p, _D, C.c_int32, C.c_double, C.c_int32, _I64, C.c_int32], C.c_int32),
    "or_distribute_cg1": ([C.c_void_p, _D, C.c_int32], None),
    "or_kinetic_energy": ([C.c_void_p], C.c_double),
    "or_image_charges": ([C.c_void_p, _D, C.c_int32, _D], None),
    "or_pcg": ([C.c_void_p, _D, _I64, _D, _D, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32], C.c_int32),
    "or_mass_matvec": ([C.c_void_p, _D, _D], None),
    "or_amg_setup": ([C.c_void_p, _I64, C.c_int32, C.c_int32], C.c_void_p),
    "or_amg_levels": ([C.c_void_p, _I64, C.c_int32], C.c_int32),
    "or_amg_free": ([C.c_void_p], None),
    "or_amg_pcg": ([C.c_void_p, C.c_void_p, _D, _I64, _D, _D, C.c_double, C.c_double, C.c_int32, C.c_int32,
                    C.c_int32], C.c_int32),
    "or_create_flux": ([C.c_void_p, _D, C.c_int32], None),
    "or_inject": ([C.c_void_p, C.c_double, C.c_uint64, C.c_uint64, _I64], C.c_int64),
    "or_n_ext_facets": ([C.c_void_p], C.c_int64),
    "or_ndof": ([C.c_void_p], C.c_int64),
    "or_next_id": ([C.c_void_p], C.c_int64),
    "or_set_next_id": ([C.c_void_p, C.c_int64], None),
    "or_exp_series": ([C.c_double], C.c_double),
    "or_philox_block": ([C.POINTER(C.c_uint32)] * 3, None),
    "or_philox_uniforms": ([C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int64, _D], None),
}
_lib = None

# table ids of or_table
T_BARY, T_PLANES, T_NBR, T_DOFS, T_VOLUME, T_DV_INV, T_ROWPTR, T_COL, T_K, T_M, T_EXT, T_BC, T_OFAC, T_CELLV = range(14)
_TDT = {T_BARY: np.float64, T_PLANES: np.float64, T_NBR: np.int64, T_DOFS: np.int64, T_VOLUME: np.float64,
        T_DV_INV: np.float64, T_ROWPTR: np.int64, T_COL: np.int64, T_K: np.float64, T_M: np.float64,
        T_EXT: np.float64, T_BC: np.int64, T_OFAC: np.float64, T_CELLV: np.int64}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "oracle.cpp")):
            build()
        L = C.CDLL(LIB)
        for k, (a, r) in _SIG.items():
            f = getattr(L, k)
            f.argtypes = a
            f.restype = r
        _lib = L
    return _lib


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_D)


def _l(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int64).ctypes.data_as(_I64)


class Oracle:
    """Mesh tables + Population<3> + stages, all on the CPU."""

    def __init__(self, mesh, eps0: float = 1.0):
        L = lib()
        self.mesh = mesh
        self.eps0 = eps0
        self._keep = [np.ascontiguousarray(mesh.coords, np.float64), np.ascontiguousarray(mesh.cells, np.int64),
                      np.ascontiguousarray(mesh.bfacets, np.int64), np.ascontiguousarray(mesh.btags, np.int32)]
        v2d = None if mesh.vertex_to_dof is None else np.ascontiguousarray(mesh.vertex_to_dof, np.int64)
        st = C.c_int32(0)
        co, ce, bf, bt = self._keep
        self.h = L.or_create(_d(co), co.shape[0], _l(ce), ce.shape[0], _l(bf), bt.ctypes.data_as(_I32), bf.shape[0],
                             _l(v2d), mesh.n_dofs, eps0, C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle mesh build failed ({st.value})")
        self.ndof = int(L.or_ndof(self.h))
        self.nc = int(mesh.cells.shape[0])
        self.n_objects = int(mesh.n_objects)
        self.species = []   # (q, m) in first-use order, like the engine

    def __del__(self):
        for h in getattr(self, "_amg", {}).values():
            lib().or_amg_free(h)
        self._amg = {}
        if getattr(self, "h", None):
            lib().or_free(self.h)
            self.h = None

    def table(self, which):
        L = lib()
        n = int(L.or_table_size(self.h, which))
        out = np.zeros(n, dtype=_TDT[which])
        L.or_table(self.h, which, out.ctypes.data_as(C.c_void_p))
        return out

    def _species(self, q, m):
        if (q, m) not in self.species:
            self.species.append((q, m))

    def locate(self, xs):
        xs = np.ascontiguousarray(xs, np.float64)
        out = np.zeros(xs.shape[0], np.int64)
        lib().or_locate(self.h, _d(xs), xs.shape[0], _l(out))
        return out

    def add_particles(self, xs, vs, q, m):
        self._species(q, m)
        xs = np.ascontiguousarray(xs, np.float64)
        vs = np.ascontiguousarray(vs, np.float64)
        return int(lib().or_add_particles(self.h, _d(xs), _d(vs), xs.shape[0], q, m))

    def num_particles(self):
        return int(lib().or_num_particles(self.h))

    def particles(self, sort=True):
        """dict of arrays x, v, q, m, cell, id (sorted by (cell, id) if sort)."""
        n = self.num_particles()
        x = np.zeros((n, 3)); v = np.zeros((n, 3)); q = np.zeros(n); m = np.zeros(n)
        cell = np.zeros(n, np.int64); pid = np.zeros(n, np.int64)
        lib().or_get_particles(self.h, _d(x), _d(v), _d(q), _d(m), _l(cell), _l(pid))
        if sort:
            o = np.lexsort((pid, cell))
            x, v, q, m, cell, pid = x[o], v[o], q[o], m[o], cell[o], pid[o]
        return dict(x=x, v=v, q=q, m=m, cell=cell, id=pid)

    def set_particles(self, p):
        n = len(p["q"])
        lib().or_set_particles(self.h, _d(p["x"]), _d(p["v"]), _d(p["q"]), _d(p["m"]), _l(p["cell"]), _l(p["id"]), n)
        for q, m in zip(p["q"], p["m"]):
            self._species(float(q), float(m))

    def efield(self, phi, E0=None):
        E = np.zeros((self.nc, 3))
        lib().or_efield_dg0(self.h, _d(phi), _d(None if E0 is None else np.asarray(E0, float)), _d(E))
        return E

    def boris(self, E, B, dt, nthreads=1):
        return float(lib().or_boris(self.h, _d(E), _d(np.asarray(B, float)), dt, nthreads))

    def accel(self, E, dt, nthreads=1):
        return float(lib().or_accel(self.h, _d(E), dt, nthreads))

    def esolver(self, phi):
        """ESolver::solve (punc/src/efield.cpp:70-75): CG1 projection of
        -grad(phi), M E_c = b_c solved directly (scipy SuperLU); [ndof][3]."""
        import scipy.sparse.linalg as spla
        b = np.zeros((self.ndof, 3))
        lib().or_esolver_rhs(self.h, _d(np.ascontiguousarray(phi, float)), _d(b))
        _, M = self.matrices()
        lu = spla.splu(M.tocsc())
        return np.ascontiguousarray(np.stack([lu.solve(b[:, c]) for c in range(3)], axis=1))

    def save_file(self, fname, binary=True):
        assert lib().or_save_population(self.h, str(fname).encode(), 1 if binary else 0) == 0

    def potential_energy(self, phi):
        return float(lib().or_potential_energy(self.h, _d(np.ascontiguousarray(phi, float))))

    def density_cg1(self, weight_e, weight_i):
        ne, ni = np.zeros(self.ndof), np.zeros(self.ndof)
        lib().or_density_cg1(self.h, weight_e, weight_i, _d(ne), _d(ni))
        return ne, ni

    def density_dg0(self, weight_e, weight_i):
        ne, ni = np.zeros(self.nc), np.zeros(self.nc)
        lib().or_density_dg0(self.h, weight_e, weight_i, _d(ne), _d(ni))
        return ne, ni

    def statistics(self):
        out = np.zeros(4)
        lib().or_statistics(self.h, _d(out))
        return out

    def accel_cg1(self, Ev, dt, nthreads=1):
        return float(lib().or_accel_cg1(self.h, _d(np.ascontiguousarray(Ev, float)), dt, nthreads))

    def boris_cg1(self, Ev, B, dt, nthreads=1):
        return float(lib().or_boris_cg1(self.h, _d(np.ascontiguousarray(Ev, float)), _d(np.asarray(B, float)), dt,
                                        nthreads))

    def move(self, dt, Ld=None, nthreads=1):
        lib().or_move(self.h, dt, _d(None if Ld is None else np.asarray(Ld, float)), nthreads)

    def update(self, objects, dt, nthreads=1, n_tags=64):
        """objects: list of dicts with bnd_id, charge, current, potential (mutated)."""
        arr = np.array([[o["bnd_id"], o["charge"], o["current"], o["potential"]] for o in objects],
                       dtype=np.float64).reshape(-1, 4)
        absorbed = np.zeros(n_tags, np.int64)
        rc = lib().or_update(self.h, _d(arr), len(objects), dt, nthreads, _l(absorbed), n_tags)
        if rc != 0:
            raise RuntimeError("oracle walk hit its step limit")
        for o, a in zip(objects, arr):
            o["charge"], o["current"] = float(a[1]), float(a[2])
        return absorbed

    def distribute_cg1(self, nthreads=1):
        rho = np.zeros(self.ndof)
        lib().or_distribute_cg1(self.h, _d(rho), nthreads)
        return rho

    def kinetic_energy(self):
        return float(lib().or_kinetic_energy(self.h))

    def image_charges(self, phi):
        out = np.zeros(max(1, self.n_objects))
        lib().or_image_charges(self.h, _d(phi), self.n_objects, _d(out))
        return out[: self.n_objects]

    # ---- Poisson ----------------------------------------------------------
    def matrices(self):
        import scipy.sparse as sp
        rp, col = self.table(T_ROWPTR), self.table(T_COL)
        K = sp.csr_matrix((self.table(T_K), col, rp), shape=(self.ndof, self.ndof))
        M = sp.csr_matrix((self.table(T_M), col, rp), shape=(self.ndof, self.ndof))
        return K, M

    def dirichlet(self, periodic=False, ext_E=(0.0, 0.0, 0.0)):
        """bc kind per dof (-1 free, 0 exterior, k object k-1) and exterior values."""
        kind = self.table(T_BC)
        if periodic:
            kind = -np.ones_like(kind)
        g = np.zeros(self.ndof)
        if not periodic and np.any(np.asarray(ext_E) != 0):
            cv = self.table(T_CELLV).reshape(-1, 4)
            dofs = self.table(T_DOFS).reshape(-1, 4)
            co = self.mesh.coords
            for c in range(cv.shape[0]):
                for i in range(4):
                    x = co[cv[c, i]]
                    g[dofs[c, i]] = ((0.0 + x[0] * ext_E[0]) + x[1] * ext_E[1]) + x[2] * ext_E[2]
        return kind, g

    def poisson_direct(self, rho, potentials=None, periodic=False, ext_E=(0.0, 0.0, 0.0)):
        """PoissonSolver::solve (punc/src/poisson.cpp:343-362) by a direct sparse
        solve of the DirichletBC-applied system: Dirichlet rows replaced by
        identity rows with b = value; periodic: b orthogonalised against the
        constant null space, solution shifted to zero mean."""
        import scipy.sparse as sp
        import scipy.sparse.linalg as sla
        K, M = self.matrices()
        b = M @ np.asarray(rho, float)
        kind, g = self.dirichlet(periodic, ext_E)
        A = K.tolil() if False else K.tocsr(copy=True)
        if periodic:
            b = b - b.mean()
            A = A.tolil()
            A[0, :] = 0
            A[0, 0] = 1.0
            b = b.copy()
            b[0] = 0.0
            x = sla.spsolve(A.tocsr(), b)
            return x - x.mean()
        vals = g.copy()
        if potentials is not None:
            for k, p in enumerate(potentials):
                vals[kind == k + 1] = p
        bc = kind >= 0
        D = sp.diags((~bc).astype(float))
        A = D @ K + sp.diags(bc.astype(float))
        b = np.where(bc, vals, b)
        return sla.spsolve(A.tocsc(), b)

    def poisson_pcg(self, rho, potentials=None, periodic=False, x0=None, rtol=1e-12, atol=1e-14, max_iter=1000,
                    nthreads=1):
        """The engine's Jacobi-PCG on the CPU (timed CPU baseline)."""
        kind, g = self.dirichlet(periodic)
        if potentials is not None:
            for k, p in enumerate(potentials):
                g[kind == k + 1] = p
        K, M = self.matrices()
        b = np.zeros(self.ndof)
        lib().or_mass_matvec(self.h, _d(np.asarray(rho, float)), _d(b))
        free = kind < 0
        bcv = np.where(kind >= 0, g, 0.0)
        b = np.where(free, b - K @ bcv, g)
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, float)
        it = lib().or_pcg(self.h, _d(b), _l(kind), _d(g), _d(x), rtol, atol, max_iter, 1 if periodic else 0, nthreads)
        if it < 0:
            raise RuntimeError("oracle PCG did not converge")
        return x, int(it)

    def poisson_amg(self, rho, potentials=None, periodic=False, x0=None, rtol=1e-12, atol=1e-14, max_iter=1000,
                    nthreads=1):
        """CG preconditioned by a smoothed-aggregation AMG V-cycle (the
        reference's solver class: PETSc + hypre AMG, punc/src/poisson.cpp:297-304)
        on the system of poisson_pcg.  The hierarchy is built on the first
        call (per periodic flag) and kept.  Returns (x, iterations)."""
        kind, g = self.dirichlet(periodic)
        if potentials is not None:
            for k, p in enumerate(potentials):
                g[kind == k + 1] = p
        key = bool(periodic)
        if not hasattr(self, "_amg"):
            self._amg = {}
        if key not in self._amg:
            h = lib().or_amg_setup(self.h, _l(kind), 1 if periodic else 0, nthreads)
            if not h:
                raise RuntimeError("oracle AMG set-up failed")
            self._amg[key] = h
        K, M = self.matrices()
        b = np.zeros(self.ndof)
        lib().or_mass_matvec(self.h, _d(np.asarray(rho, float)), _d(b))
        free = (kind < 0) | bool(periodic)
        bcv = np.where(free, 0.0, g)
        b = np.where(free, b - K @ bcv, g)
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, float)
        it = lib().or_amg_pcg(self.h, self._amg[key], _d(b), _l(kind), _d(g), _d(x), rtol, atol, max_iter,
                              1 if periodic else 0, nthreads)
        if it < 0:
            raise RuntimeError("oracle AMG-PCG did not converge")
        return x, int(it)

    def amg_levels(self, periodic=False):
        rows = np.zeros(16, np.int64)
        n = lib().or_amg_levels(self._amg[bool(periodic)], _l(rows), 16)
        return rows[:n].tolist()

    # ---- injection ------------------------------------------------------------
    def create_flux(self, species):
        """species: list of dicts q, m, n, vth, vd, (vdf_range) in engine-id order."""
        arr = np.zeros((len(species), 9))
        for k, s in enumerate(species):
            arr[k, :8] = [s["q"], s["m"], s["n"], s["vth"], *s.get("vd", (0.0, 0.0, 0.0)), s.get("vdf_range", 5.0)]
            self._species(s["q"], s["m"])
        lib().or_create_flux(self.h, _d(arr), len(species))

    def inject(self, dt, seed, step):
        counts = np.zeros(8, np.int64)
        n = lib().or_inject(self.h, dt, seed, step, _l(counts))
        return int(n), counts


class CircuitCM:
    """CircuitCM (punc/src/object_CM.cpp:135-376) over an oracle Poisson solve."""

    def __init__(self, oracle: Oracle, vsources, isources, dt, solve):
        n = oracle.n_objects
        self.n, self.dt = n, dt
        self.vsources = [tuple(v) for v in vsources]
        self.isources = [tuple(v) for v in isources]
        self.solve = solve     # solve(rho or None, potentials) -> phi
        cap = np.zeros((n, n))
        for j in range(n):
            pot = np.zeros(n); pot[j] = 1.0
            phi = solve(None, pot, laplace=True)
            cap[:, j] = oracle.image_charges(phi)
        self.cap = cap
        self.inv_cap = np.linalg.inv(cap)
        self.groups = self._groups(list(self.vsources), n)
        self.fixed_voltage = []
        for a, b, _ in self.vsources:
            if a == -1:
                tmp = [b]; node = b
                for a2, b2, _v in self.vsources:
                    if a2 == node:
                        tmp.append(b2); node = b2
                self.fixed_voltage.append(tmp)
        self.circuit_vector = np.zeros(2 * n)
        for a, b, v in self.vsources:
            self.circuit_vector[b] = v
        Mx = np.zeros((2 * n, 2 * n))
        for a, b, _ in self.vsources:
            Mx[b, b] = 1.0
            if a != -1:
                Mx[b, a] = -1.0
        ic = self.inv_cap
        for g in self.groups:
            for v in g:
                Mx[n + g[0], n + v] = 1.0
            Mx[g[0], g[0]] = 1.0
            for v in g:
                Mx[g[0], n + v] = -1.0 * ic[g[0], v]
            for j in g[1:]:
                Mx[n + j, j] = 1.0
                for v in g:
                    Mx[n + j, n + v] = -1.0 * ic[j, v]
        for fv in self.fixed_voltage:
            for a in fv:
                Mx[n + a, a] = 1.0
                for b in fv:
                    Mx[n + a, n + b] = -1.0 * ic[a, b]
        self.inv_circuit = np.linalg.inv(Mx)
        self.oracle = oracle

    @staticmethod
    def _groups(vs, n):
        def collect(vs, node, group):
            group.append(node)
            i = 0
            while i < len(vs):
                a, b, v = vs[i]
                if a == node:
                    vs.pop(i); collect(vs, b, group)
                elif b == node:
                    vs.pop(i); collect(vs, a, group)
                else:
                    i += 1
        nodes = list(range(n))
        groups = []
        while vs:
            g = []
            collect(vs, vs[0][0], g)
            groups.append(g)
        for g in groups:
            for v in g:
                if v != -1 and v in nodes:
                    nodes.remove(v)
        groups = [g for g in groups if -1 not in g]
        groups += [[v] for v in nodes]
        return groups

    def solve_circuit(self, rho, objects):
        """PoissonSolver::solve_circuit with CM (punc/src/poisson.cpp:364-376)."""
        n = self.n
        for a, b, v in self.isources:
            dQ = v * self.dt
            if a != -1:
                objects[a]["charge"] -= dQ
            if b != -1:
                objects[b]["charge"] += dQ
        for o in objects:
            o["potential"] = 0.0
        phi = self.solve(rho, np.zeros(n))
        img = self.oracle.image_charges(phi)
        cv = self.circuit_vector
        ic = self.inv_cap
        for g in self.groups:
            cv[n + g[0]] = sum(objects[v]["charge"] for v in g)
        for g in self.groups:
            cv[g[0]] = sum(ic[g[0], v] * img[v] for v in g)
            for j in g[1:]:
                cv[n + j] = sum(ic[j, v] * img[v] for v in g)
        for fv in self.fixed_voltage:
            for a in fv:
                cv[n + a] = sum(ic[a, b] * img[b] for b in fv)
        pots = np.zeros(n)
        for i in range(n):
            objects[i]["potential"] = float(self.inv_circuit[i] @ cv)
            objects[i]["charge"] = float(self.inv_circuit[n + i] @ cv)
            pots[i] = objects[i]["potential"]
        return self.solve(rho, pots), img


class PeriodicPoisson:
    """y = A^+ P b for the periodic P1 stiffness A (constant null space, P the
    mean removal): the oracle's Jacobi-PCG on P b to a relative residual of
    1e-13, then the mean removed from the solution (poisson.cpp:343-362 with
    the null space orthogonalised out)."""

    def __init__(self, oracle: Oracle, nthreads=1):
        self.o = oracle
        self.kind = -np.ones(oracle.ndof, np.int64)
        self.g = np.zeros(oracle.ndof)
        self.nthreads = nthreads

    def __call__(self, b):
        b = np.ascontiguousarray(b, float)
        x = np.zeros(self.o.ndof)
        it = lib().or_pcg(self.o.h, _d(b), _l(self.kind), _d(self.g), _d(x), 1e-13, 0.0, 100000, 1, self.nthreads)
        if it < 0:
            raise RuntimeError("oracle PCG did not converge")
        return x - x.mean()


def langmuir_adjoint(mesh, x0, v0, q, m, E0, dt, n_steps, target, Ld, first_step=True, nthreads=1):
    """Loss ||rho_K - target||^2 of K periodic steps (CG1 deposit, P1 Poisson,
    DG0 field plus the uniform E0, Boris push with B = 0, periodic move) and its
    gradients by a reverse sweep with the cells fixed from the forward pass.
    Not a reference algorithm (the reference has no adjoint): the derivative of
    the stages restated above (distribute_cg1: punc/src/distributor.cpp,
    efield_DG0: punc/src/efield.cpp, boris: punc/include/punc/pusher.h,
    move_periodic: pusher.h), checked against jump-free finite differences.
    Reverse step n: vbar += dt xbar; Ebar_c = sum_{p in c} coef vbar_p;
    E0bar += sum_p coef vbar_p; phibar_k -= Ebar_c . grad lambda_k(c);
    rhobar = M A^+ P phibar; xbar_p += q sum_i dv_inv_i rhobar_i grad lambda_i.
    Returns (loss, grad_v0 [n][3], grad_E0 [3], grad_x0 [n][3]), rows by
    particle id (insertion order)."""
    o = Oracle(mesh)
    K, M = o.matrices()
    solve = PeriodicPoisson(o, nthreads)
    n = o.add_particles(x0, v0, q, m)
    if n != len(x0):
        raise ValueError("langmuir_adjoint: a particle lies outside the mesh")
    bary = o.table(T_BARY).reshape(-1, 12)
    dofs = o.table(T_DOFS).reshape(-1, 4)
    dv_inv = o.table(T_DV_INV)
    G = np.zeros((o.nc, 4, 3))
    for i in range(3):
        G[:, i, :] = bary[:, 4 * i + 1:4 * i + 4]
    G[:, 3, :] = -G[:, :3, :].sum(axis=1)

    def cells_by_id():
        p = o.particles(sort=False)
        out = np.empty(n, np.int64)
        out[p["id"]] = p["cell"]
        return out

    cells = []
    for k in range(n_steps):
        cells.append(cells_by_id())
        phi = solve(M @ o.distribute_cg1(nthreads))
        E = o.efield(phi, E0)
        o.boris(E, (0.0, 0.0, 0.0), 0.5 * dt if (first_step and k == 0) else dt, nthreads)
        o.move(dt, Ld, nthreads)
        o.update([], dt, nthreads)
    cells.append(cells_by_id())
    rho = o.distribute_cg1(nthreads)
    loss = float(np.sum((rho - target) ** 2))

    def deposit_adjoint(rhobar, c):
        # per cell sum_i dv_inv_i rhobar_i grad lambda_i, gathered per particle
        per_cell = np.einsum("ci,cij->cj", dv_inv[dofs] * rhobar[dofs], G)
        return q * per_cell[c]

    xb = deposit_adjoint(2.0 * (rho - target), cells[n_steps])
    vb = np.zeros((n, 3))
    e0b = np.zeros(3)
    for k in range(n_steps - 1, -1, -1):
        coef = (0.5 * dt if (first_step and k == 0) else dt) * (q / m)
        vb += dt * xb
        Eb = np.stack([np.bincount(cells[k], weights=coef * vb[:, j], minlength=o.nc) for j in range(3)], axis=1)
        e0b += coef * vb.sum(axis=0)
        phib = np.bincount(dofs.ravel(), weights=-np.einsum("cj,cij->ci", Eb, G).ravel(), minlength=o.ndof)
        rhob = M @ solve(phib)
        xb += deposit_adjoint(rhob, cells[k])
    return loss, vb, e0b, xb


def langmuir_loss(mesh, x0, v0, q, m, E0, dt, n_steps, target, Ld, first_step=True, nthreads=1):
    """The forward of langmuir_adjoint alone (for finite differences)."""
    o = Oracle(mesh)
    _, M = o.matrices()
    solve = PeriodicPoisson(o, nthreads)
    o.add_particles(x0, v0, q, m)
    for k in range(n_steps):
        phi = solve(M @ o.distribute_cg1(nthreads))
        o.boris(o.efield(phi, E0), (0.0, 0.0, 0.0), 0.5 * dt if (first_step and k == 0) else dt, nthreads)
        o.move(dt, Ld, nthreads)
        o.update([], dt, nthreads)
    return float(np.sum((o.distribute_cg1(nthreads) - target) ** 2))
