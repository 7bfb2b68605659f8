"""Python front end with the names and call order of the PUNC++ particle path.

A time loop written against the reference (interaction/interaction.cpp:342-480):

    distribute_cg1(pop, rho, dv_inv)
    poisson.solve_circuit(phi, rho, mesh, objects, circuit)
    esolver.solve(E, phi)                 # EFieldDG0
    KE = boris(pop, E, B, dt)             # or accel(pop, E, dt)
    move(pop, dt)
    pop.update(objects, dt)
    inject_particles(pop, species, mesh.exterior_facets, dt)

runs unchanged on these classes; every call goes through the C ABI of
libpunc_gpu.so into device-resident state.  Fields (E, rho, phi) live on the
device inside the Population's engine handle; Function objects are views that
download on .vector().
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .meshgen import MeshArrays


class Mesh:
    """Host mesh tables (pg_mesh_build): the reference Mesh plus the tables its
    Population constructor derives (punc/src/mesh.cpp:41-60)."""

    dim = 3
    ext_bnd_id = 1

    def __init__(self, arrays: MeshArrays, eps0: float = 1.0):
        lib = L.load()
        self.arrays = arrays
        self.eps0 = eps0
        self._keep = [np.ascontiguousarray(arrays.coords, np.float64), np.ascontiguousarray(arrays.cells, np.int64),
                      np.ascontiguousarray(arrays.bfacets, np.int64), np.ascontiguousarray(arrays.btags, np.int32)]
        v2d = None if arrays.vertex_to_dof is None else np.ascontiguousarray(arrays.vertex_to_dof, np.int64)
        self._keep.append(v2d)
        co, ce, bf, bt, _ = self._keep
        d = L.MeshDesc(co.shape[0], L.dptr(co), ce.shape[0], L.i64ptr(ce), bf.shape[0], L.i64ptr(bf),
                       L.i32ptr(bt), arrays.n_dofs, L.i64ptr(v2d))
        h = C.c_void_p()
        L.check(lib.pg_mesh_build(C.byref(d), eps0, C.byref(h)))
        self.handle = h
        self.num_objects = int(arrays.n_objects)
        self.Ld = arrays.Ld

    def table(self, which: int) -> np.ndarray:
        ptr = C.c_void_p()
        n = C.c_int64()
        L.check(L.load().pg_mesh_array(self.handle, which, C.byref(ptr), C.byref(n)))
        dt = L._TABLE_DTYPE[which]
        if n.value == 0:
            return np.zeros(0, dtype=dt)
        buf = (C.c_char * (n.value * np.dtype(dt).itemsize)).from_address(ptr.value)
        return np.frombuffer(buf, dtype=dt).copy()

    @property
    def exterior_facets(self) -> np.ndarray:
        return self.table(L.T_EXT_FACETS).reshape(-1, 14)

    @property
    def n_dofs(self) -> int:
        return int(self.arrays.n_dofs)

    @property
    def num_cells(self) -> int:
        return int(self.arrays.n_cells)

    def volume(self) -> float:
        """Mesh::volume (punc/src/mesh.cpp:147-170): the cell volumes summed in
        cell order, as the assembly of the form 1 dx accumulates them."""
        vol = self.table(L.T_VOLUME)
        return float(np.cumsum(vol)[-1]) if len(vol) else 0.0

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            L.load().pg_mesh_free(h)
            self.handle = None


@dataclass
class Object:
    """Reference Object (punc/include/punc/object.h:80-130)."""
    bnd_id: int
    charge: float = 0.0
    current: float = 0.0
    potential: float = 0.0

    def set_potential(self, p: float):
        self.potential = p

    def get_potential(self) -> float:
        return self.potential


def _objects_in(objects):
    arr = (L.Object * max(1, len(objects)))()
    for k, o in enumerate(objects):
        arr[k] = L.Object(o.bnd_id, o.charge, o.current, o.potential)
    return arr


def _objects_out(arr, objects):
    for k, o in enumerate(objects):
        o.charge, o.current, o.potential = arr[k].charge, arr[k].current, arr[k].potential


class ParticleAmountType(enum.IntEnum):
    """How the amount of simulation particles is given to Species.from_physical
    (punc/include/punc/population.h:50-55)."""
    in_total = 0       # total number of simulation particles
    per_cell = 1       # simulation particles per cell
    per_volume = 2     # simulation particles per volume
    phys_per_sim = 3   # physical particles per simulation particle


@dataclass
class Species:
    """Maxwellian species of simulation particles (punc/src/population.cpp:41-70):
    q, m and n of a simulation particle, the velocity distribution's vth, drift
    and range; weight (physical particles per simulation particle), num (the
    initial number of simulation particles) and debye (the Debye length) as
    the reference's constructor derives them in from_physical."""
    q: float
    m: float
    n: float = 0.0
    vth: float = 0.0
    vd: tuple = (0.0, 0.0, 0.0)
    vdf_range: float = 5.0
    weight: float = 1.0
    num: int = 0
    debye: float = 0.0

    @classmethod
    def from_physical(cls, charge: float, mass: float, density: float, amount: float, amount_type, mesh: Mesh,
                      vth: float = 0.0, vd=(0.0, 0.0, 0.0), vdf_range: float = 5.0, eps0: float | None = None):
        """Species::Species (punc/src/population.cpp:41-70) with a Maxwellian
        velocity distribution (Maxwellian::debye, punc/src/distributions.cpp:74-77):
        the amount becomes physical particles per simulation particle by the
        reference's chain of steps (per cell -> in total -> per volume -> weight),
        and the physical charge, mass and density scale by it."""
        t = ParticleAmountType(amount_type)
        volume = mesh.volume()
        a = float(amount)
        if t == ParticleAmountType.per_cell:
            a *= mesh.num_cells
        if t in (ParticleAmountType.per_cell, ParticleAmountType.in_total):
            a /= volume
        if t != ParticleAmountType.phys_per_sim:
            a = density / a
        q, m, n = charge * a, mass * a, density / a
        e0 = mesh.eps0 if eps0 is None else eps0
        return cls(q, m, n=n, vth=vth, vd=tuple(vd), vdf_range=vdf_range, weight=a, num=int(n * volume),
                   debye=math.sqrt(e0 * m / (n * q * q)) * vth)


def min_plasma_period(species, eps0: float) -> float:
    """min_plasma_period (punc/src/population.cpp:72-80): 2 pi over the largest
    plasma frequency sqrt(q^2 n / (eps0 m)) of the species."""
    wp_max = 0.0
    for s in species:
        wp = math.sqrt(s.q * s.q * s.n / (eps0 * s.m))
        if wp > wp_max:
            wp_max = wp
    return 2 * math.pi / wp_max


class Population:
    """Population<3> on the device (punc/include/punc/population.h:236-308)."""

    g_dim = 3

    def __init__(self, mesh: Mesh, precision: int = L.PG_FP64, periodic: bool = False, capacity: int = 0,
                 max_walk_steps: int = 0, sort_interval: int = 0, pcg_rtol: float = 0.0, pcg_atol: float = 0.0,
                 pcg_max_iter: int = 0, warm_start: int = 1, ext_E=(0.0, 0.0, 0.0),
                 circuit_resolve: bool = False, pcg_precision: int = 0, pcg_precond: int = 0):
        lib = L.load()
        self.mesh = mesh
        cfg = L.Config(precision, 1 if periodic else 0, mesh.eps0, capacity, max_walk_steps, sort_interval,
                       pcg_rtol, pcg_atol, pcg_max_iter, int(warm_start), (C.c_double * 3)(*ext_E),
                       1 if circuit_resolve else 0, pcg_precision, pcg_precond)
        h = C.c_void_p()
        L.check(lib.pg_create(mesh.handle, C.byref(cfg), C.byref(h)))
        self.handle = h
        self.num_cells = int(mesh.arrays.n_cells)
        self.ndof = mesh.n_dofs
        self.periodic = periodic

    def close(self):
        h = getattr(self, "handle", None)
        if h:
            L.load().pg_destroy(h)
            self.handle = None

    def __del__(self):
        self.close()

    def add_particles(self, xs, vs, q: float, m: float) -> int:
        xs = np.ascontiguousarray(xs, np.float64).reshape(-1, 3)
        vs = np.ascontiguousarray(vs, np.float64).reshape(-1, 3)
        n = C.c_int64()
        L.check(L.load().pg_add_particles(self.handle, L.dptr(xs), L.dptr(vs), xs.shape[0], q, m, C.byref(n)))
        return n.value

    def locate(self, xs) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.float64).reshape(-1, 3)
        out = np.zeros(xs.shape[0], np.int64)
        L.check(L.load().pg_locate(self.handle, L.dptr(xs), xs.shape[0], L.i64ptr(out)))
        return out

    def relocate(self, xs, cells, fast: bool = True, with_crossings: bool = False):
        """relocate_fast (fast) or relocate / relocate_stat
        (punc/include/punc/population.h:454-569) of points xs from the given
        cells: the final cell or -tag per point, and the facets crossed."""
        xs = np.ascontiguousarray(xs, np.float64).reshape(-1, 3)
        c0 = np.ascontiguousarray(cells, np.int64).reshape(-1)
        out = np.zeros(len(c0), np.int64)
        cr = np.zeros(len(c0), np.int32)
        L.check(L.load().pg_relocate(self.handle, L.dptr(xs), L.i64ptr(c0), len(c0), 0 if fast else 1,
                                     L.i64ptr(out), cr.ctypes.data_as(C.POINTER(C.c_int32))))
        return (out, cr) if with_crossings else out

    def _counts(self):
        t, ng, ps = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(L.load().pg_num_particles(self.handle, C.byref(t), C.byref(ng), C.byref(ps)))
        return t.value, ng.value, ps.value

    def num_of_particles(self) -> int:
        return self._counts()[0]

    def num_of_negatives(self) -> int:
        return self._counts()[1]

    def num_of_positives(self) -> int:
        return self._counts()[2]

    def save_file(self, fname: str, binary: bool = True):
        """Population::save_file (punc/include/punc/population.h:806-837)."""
        L.check(L.load().pg_population_save(self.handle, str(fname).encode(), 1 if binary else 0))

    def load_file(self, fname: str, binary: bool = True) -> int:
        """Population::load_file (punc/include/punc/population.h:839-878); returns
        the number of particles added."""
        n = C.c_int64()
        L.check(L.load().pg_population_load(self.handle, str(fname).encode(), 1 if binary else 0, C.byref(n)))
        return n.value

    def statistics(self) -> np.ndarray:
        """Population::statistics (punc/include/punc/population.h:746-805): mean
        speed and sample standard deviation of the negative, then the positive
        particles."""
        out = np.zeros(4)
        L.check(L.load().pg_statistics(self.handle, L.dptr(out)))
        return out

    def particles(self, fields=("x", "v", "q", "m", "cell", "id")) -> dict:
        """Live particles ordered by (cell, id): x, v, q, m, cell, id (only
        the named fields cross to the host)."""
        lib = L.load()
        n = C.c_int64()
        L.check(lib.pg_get_particles(self.handle, 0, None, None, None, None, None, None, C.byref(n)))
        k = n.value
        shapes = {"x": (k, 3), "v": (k, 3), "q": (k,), "m": (k,), "cell": (k,), "id": (k,)}
        out = {f: np.zeros(shapes[f], np.int64 if f in ("cell", "id") else np.float64) for f in fields}
        ptr = {f: (L.i64ptr(a) if f in ("cell", "id") else L.dptr(a)) for f, a in out.items()}
        L.check(lib.pg_get_particles(self.handle, k, ptr.get("x"), ptr.get("v"), ptr.get("q"), ptr.get("m"),
                                     ptr.get("cell"), ptr.get("id"), C.byref(n)))
        return out

    def update(self, objects, dt: float):
        arr = _objects_in(objects)
        L.check(L.load().pg_update(self.handle, arr, len(objects), dt))
        _objects_out(arr, objects)

    def sort(self):
        L.check(L.load().pg_sort(self.handle))

    def status(self):
        code, idx = C.c_int32(), C.c_int64()
        L.check(L.load().pg_status_detail(self.handle, C.byref(code), C.byref(idx)))
        return code.value, idx.value


class Function:
    """A field of the Population's engine: 'E' (DG0 vector), 'E_cg1' (CG1
    vector, [Ndof][3]), 'rho' or 'phi' (CG1)."""

    def __init__(self, pop: Population, kind: str):
        assert kind in ("E", "E_cg1", "rho", "phi")
        self.pop, self.kind = pop, kind

    def vector(self) -> np.ndarray:
        lib = L.load()
        if self.kind == "E":
            out = np.zeros((self.pop.num_cells, 3))
            L.check(lib.pg_get_efield(self.pop.handle, L.dptr(out)))
        elif self.kind == "E_cg1":
            out = np.zeros((self.pop.ndof, 3))
            L.check(lib.pg_get_efield_cg1(self.pop.handle, L.dptr(out)))
        else:
            out = np.zeros(self.pop.ndof)
            fn = lib.pg_get_rho if self.kind == "rho" else lib.pg_get_phi
            L.check(fn(self.pop.handle, L.dptr(out)))
        return out

    def set_local(self, values):
        v = np.ascontiguousarray(values, np.float64)
        lib = L.load()
        if self.kind == "E":
            L.check(lib.pg_set_efield(self.pop.handle, L.dptr(v.reshape(-1, 3))))
        elif self.kind == "E_cg1":
            L.check(lib.pg_set_efield_cg1(self.pop.handle, L.dptr(v.reshape(-1, 3))))
        elif self.kind == "rho":
            L.check(lib.pg_set_rho(self.pop.handle, L.dptr(v)))
        else:
            L.check(lib.pg_efield_dg0(self.pop.handle, L.dptr(v)))  # uploads phi and refreshes E


def accel(pop: Population, E: Function, dt: float) -> float:
    """accel with a DG0 field (punc/include/punc/pusher.h:66-130)."""
    ke = C.c_double()
    L.check(L.load().pg_accel(pop.handle, dt, C.byref(ke)))
    return ke.value


def boris(pop: Population, E: Function, B, dt: float) -> float:
    """boris with a DG0 field and uniform B (punc/include/punc/pusher.h:397-510)."""
    b = np.ascontiguousarray(B, np.float64)
    ke = C.c_double()
    L.check(L.load().pg_boris(pop.handle, L.dptr(b), dt, C.byref(ke)))
    return ke.value


def accel_cg1(pop: Population, E: Function, dt: float) -> float:
    """accel_cg1 with the CG1 field (punc/include/punc/pusher.h:154-201)."""
    ke = C.c_double()
    L.check(L.load().pg_accel_cg1(pop.handle, dt, C.byref(ke)))
    return ke.value


def boris_cg1(pop: Population, E: Function, B, dt: float) -> float:
    """boris_cg1 with the CG1 field and uniform B (punc/include/punc/pusher.h:282-372)."""
    b = np.ascontiguousarray(B, np.float64)
    ke = C.c_double()
    L.check(L.load().pg_boris_cg1(pop.handle, L.dptr(b), dt, C.byref(ke)))
    return ke.value


def move(pop: Population, dt: float):
    L.check(L.load().pg_move(pop.handle, dt))


def move_periodic(pop: Population, dt: float, Ld):
    Ld = np.ascontiguousarray(Ld, np.float64)
    L.check(L.load().pg_move_periodic(pop.handle, dt, L.dptr(Ld)))


def element_volume(mesh: Mesh, voronoi: bool = True) -> np.ndarray:
    """element_volume (punc/src/distributor.cpp:35-69): per dof, (d + 1) over
    the volume of its cells (voronoi) or one over that volume.  The engine
    keeps the first as a mesh table; the second is it divided by 4 (exact)."""
    dv = mesh.table(L.T_DV_INV)
    return dv if voronoi else dv / 4.0


def distribute_cg1(pop: Population, rho: Function | None = None, dv_inv=None) -> np.ndarray:
    """distribute_cg1 (punc/include/punc/distributor.h:168-210); dv_inv is the
    engine's element_volume table, so the argument is accepted and unused."""
    out = np.zeros(pop.ndof)
    L.check(L.load().pg_distribute_cg1(pop.handle, L.dptr(out)))
    return out


def absorbed_counts(pop: Population, n_tags: int = 0):
    """The last update's absorbed particles per boundary tag and species
    (pg_absorbed_counts; Population::update sums them over the species into
    each object's current): (counts [n_tags][n_species], q [n_species],
    m [n_species]); n_tags 0: exterior and every object tag."""
    lib = L.load()
    ns = C.c_int32()
    L.check(lib.pg_absorbed_counts(pop.handle, None, 0, 0, None, None, C.byref(ns)))
    k = ns.value
    t = n_tags or pop.mesh.num_objects + 2
    counts = np.zeros((t, k), np.int64)
    q, m = np.zeros(k), np.zeros(k)
    L.check(lib.pg_absorbed_counts(pop.handle, L.i64ptr(counts), t, k, L.dptr(q), L.dptr(m), C.byref(ns)))
    return counts, q, m


def kinetic_energy(pop: Population) -> float:
    ke = C.c_double()
    L.check(L.load().pg_kinetic_energy(pop.handle, C.byref(ke)))
    return ke.value


def particle_potential_energy_cg1(pop: Population, phi: Function) -> float:
    """particle_potential_energy_cg1 (punc/include/punc/diagnostics.h:379-412)
    with the engine's current potential."""
    pe = C.c_double()
    L.check(L.load().pg_potential_energy(pop.handle, C.byref(pe)))
    return pe.value


def density_cg1(pop: Population, weight_e: float, weight_i: float):
    """density_cg1 (punc/include/punc/diagnostics.h:492-555): (ne, ni) per dof."""
    ne, ni = np.zeros(pop.ndof), np.zeros(pop.ndof)
    L.check(L.load().pg_density_cg1(pop.handle, weight_e, weight_i, L.dptr(ne), L.dptr(ni)))
    return ne, ni


def density_dg0(pop: Population, weight_e: float, weight_i: float):
    """density_dg0 (punc/include/punc/diagnostics.h:433-465): (ne, ni) per cell."""
    ne, ni = np.zeros(pop.num_cells), np.zeros(pop.num_cells)
    L.check(L.load().pg_density_dg0(pop.handle, weight_e, weight_i, L.dptr(ne), L.dptr(ni)))
    return ne, ni


class State:
    """State (punc/src/diagnostics.cpp:40-68): the resume file holding the next
    step number, the time and each object's charge and current, written with
    the default stream format (six significant digits)."""

    def __init__(self, fname: str):
        self.fname = str(fname)

    def save(self, n: int, t: float, objects):
        with open(self.fname, "w") as f:
            f.write(f"{n + 1}\t{t:g}\t")
            for o in objects:
                f.write(f"{o.charge:g}\t{o.current:g}\n")

    def load(self, objects):
        """Returns (n, t) and sets each object's charge and current from the
        first line, as the reference parses it (objects whose values are not
        on that line get 0)."""
        with open(self.fname) as f:
            tok = f.readline().split()
        n, t = int(tok[0]), float(tok[1])
        vals = [float(x) for x in tok[2:]]
        for k, o in enumerate(objects):
            o.charge = vals[2 * k] if 2 * k < len(vals) else 0.0
            o.current = vals[2 * k + 1] if 2 * k + 1 < len(vals) else 0.0
        return n, t


class History:
    """History (punc/src/diagnostics.cpp:70-140, punc/include/punc/diagnostics.h:
    119-168): the history.dat preamble and one tab-separated row per step, the
    step as an integer and the rest in scientific notation with 16 digits after
    the point (std::setprecision(digits10 + 1) << std::scientific), as the
    reference writes them."""

    def __init__(self, fname: str, objects, dim: int = 3, stats: bool = False, continue_simulation: bool = False):
        self.stats = stats
        self.f = open(fname, "a" if continue_simulation else "w")
        if not continue_simulation:
            n = len(objects)
            self.f.write("#:xaxis\tt\n")
            self.f.write("#:name\tn\tt\tne\tni\tKE\tPE" + "".join(f"\tV[{i}]\tI[{i}]\tQ[{i}]" for i in range(n)))
            if stats:
                self.f.write("\tmean_e\tstdev_e\tmean_i\tstdev_i")
            self.f.write("\n")
            self.f.write('#:long\ttimestep\ttime\t"number of electrons"\t"number of ions"\t"kinetic energy"\t'
                         '"potential energy"' + "\tvoltage\tcurrent\tcharge" * n)
            if stats:
                self.f.write("\tmean velocity of electrons\tstandard deviation of electron velocities"
                             "\tmean velocity of ions\tstandard deviation of ion velocities")
            self.f.write("\n")
            unit_i = {1: "A/m**2", 2: "A/m", 3: "A"}.get(dim, "")
            self.f.write("#:units\t1\ts\tm**(-3)\tm**(-3)\tJ\tJ" + f"\tV\t{unit_i}\tC" * n)
            if stats:
                self.f.write("\tm/s\tm/s\tm/s\tm/s")
            self.f.write("\n")

    @staticmethod
    def _fmt(x: float) -> str:
        return f"{x:.16e}"

    def save(self, n: int, t: float, num_e: float, num_i: float, KE: float, PE: float, objects, pop=None):
        row = f"{n}\t" + "\t".join(self._fmt(v) for v in (t, num_e, num_i, KE, PE))
        for o in objects:
            row += f"\t{self._fmt(o.potential)}\t{self._fmt(o.current)}\t{self._fmt(o.charge)}"
        if self.stats:
            row += "".join(f"\t{self._fmt(v)}" for v in pop.statistics())
        self.f.write(row + "\n")

    def close(self):
        self.f.close()


class EFieldDG0:
    """EFieldDG0 (punc/src/efield.cpp:77-99)."""

    def solve(self, E: Function, phi: Function):
        L.check(L.load().pg_efield_dg0(E.pop.handle, None))


class ESolver:
    """ESolver (punc/src/efield.cpp:41-75): CG1 projection of -grad(phi)."""

    def __init__(self, pop: Population):
        self.pop = pop
        self.last_info = None

    def solve(self, E: Function, phi: Function) -> np.ndarray:
        info = L.SolveInfo()
        L.check(L.load().pg_esolver_solve(self.pop.handle, None, C.byref(info)))
        self.last_info = info
        return E.vector()


class CircuitCM:
    """CircuitCM (punc/src/object_CM.cpp:135-197): capacitance matrix at set-up."""

    def __init__(self, pop: Population, objects, vsources=(), isources=(), dt: float = 1.0):
        vs = (L.Source * max(1, len(vsources)))(*[L.Source(int(a), int(b), float(v)) for a, b, v in vsources])
        iss = (L.Source * max(1, len(isources)))(*[L.Source(int(a), int(b), float(v)) for a, b, v in isources])
        L.check(L.load().pg_circuit_cm_setup(pop.handle, vs, len(vsources), iss, len(isources), dt))
        self.pop = pop
        self.correction_required = True

    def inv_capacitance(self) -> np.ndarray:
        n = self.pop.mesh.num_objects
        out = np.zeros(n * n)
        L.check(L.load().pg_get_capacitance(self.pop.handle, L.dptr(out)))
        return out.reshape(n, n)


class PoissonSolver:
    """PoissonSolver (punc/src/poisson.cpp:260-385) on the device."""

    def __init__(self, pop: Population, objects=(), circuit: CircuitCM | None = None):
        self.pop = pop
        self.last_info = None

    def solve(self, phi: Function, rho: Function, objects=(), circuit=None) -> np.ndarray:
        arr = _objects_in(objects)
        info = L.SolveInfo()
        L.check(L.load().pg_poisson_solve(self.pop.handle, arr, len(objects), None, C.byref(info)))
        self.last_info = info
        return phi.vector()

    def solve_circuit(self, phi: Function, rho: Function, mesh, objects, circuit) -> np.ndarray:
        arr = _objects_in(objects)
        info = L.SolveInfo()
        L.check(L.load().pg_solve_circuit(self.pop.handle, arr, len(objects), None, C.byref(info)))
        _objects_out(arr, objects)
        self.last_info = info
        return phi.vector()


def create_flux(pop: Population, species):
    """create_flux (punc/src/injector.cpp:104-171), Maxwellian species."""
    arr = (L.Species * max(1, len(species)))()
    for k, s in enumerate(species):
        arr[k] = L.Species(s.q, s.m, s.n, s.vth, (C.c_double * 3)(*s.vd), s.vdf_range)
    L.check(L.load().pg_create_flux(pop.handle, arr, len(species)))


def load_particles(pop: Population, species, seed: int = 0, batch: int = 1 << 20) -> list:
    """load_particles (punc/include/punc/injector.h:244-278): for each
    species its num particles at positions uniform over the mesh (rejection
    sampling in the cube [min coordinate, max coordinate]^3 of UniformPosition,
    punc/include/punc/distributions.h:186-230, a point kept when it lies in a
    cell) with Maxwellian velocities (vd + vth N(0, 1) per component).  The
    reference's generator is unseeded; this one is numpy's, seeded.  Returns
    the number added per species."""
    rng = np.random.default_rng(seed)
    co = pop.mesh.arrays.coords
    lo, hi = float(co.min()), float(co.max())
    added = []
    for s in species:
        need, xs = int(s.num), []
        got = 0
        while got < need:
            pts = lo + (hi - lo) * rng.random((max(batch, 2 * (need - got)), 3))
            pts = pts[pop.locate(pts) >= 0][: need - got]
            xs.append(pts)
            got += len(pts)
        x = np.concatenate(xs) if xs else np.zeros((0, 3))
        v = np.asarray(s.vd, float) + s.vth * rng.standard_normal((need, 3))
        added.append(pop.add_particles(x, v, s.q, s.m))
    return added


def inject_particles(pop: Population, species, facets, dt: float, seed: int = 0, step: int = 0) -> int:
    """inject_particles (punc/include/punc/injector.h:157-232); create_flux must
    have been called for these species."""
    n = C.c_int64()
    L.check(L.load().pg_inject(pop.handle, dt, seed, step, C.byref(n)))
    return n.value


def step(pop: Population, objects, dt: float, B=(0.0, 0.0, 0.0), first_step=False, use_accel=False, Ld=None,
         inject=False, seed=0, step_no=0, E0=(0.0, 0.0, 0.0), efield_cg1=False,
         potential_energy=False) -> L.StepResult:
    """One fused timestep in the order of interaction.cpp:342-480 (efield_cg1:
    ESolver + accel_cg1/boris_cg1, else EFieldDG0 + accel/boris);
    potential_energy: also particle_potential_energy_cg1 of the particles at
    the step's start in the step's potential (res.PE), as the time loop
    records it."""
    a = L.StepArgs(dt, (C.c_double * 3)(*B), 1 if first_step else 0, 1 if use_accel else 0,
                   0 if Ld is None else 1, (C.c_double * 3)(*(Ld if Ld is not None else (0.0, 0.0, 0.0))),
                   1 if inject else 0, seed, step_no, (C.c_double * 3)(*E0), 1 if efield_cg1 else 0,
                   1 if potential_energy else 0)
    arr = _objects_in(objects)
    res = L.StepResult()
    L.check(L.load().pg_step(pop.handle, C.byref(a), arr, len(objects), C.byref(res)))
    _objects_out(arr, objects)
    return res


def run_steps(pop: Population, objects, dt: float, n_steps: int, B=(0.0, 0.0, 0.0), first_step=False,
              use_accel=False, Ld=None, inject=False, seed=0, step_no=0, E0=(0.0, 0.0, 0.0), efield_cg1=False,
              use_graph=True):
    """n_steps fused timesteps with the bookkeeping on the device (one host
    synchronisation at the end), optionally replaying a captured CUDA graph;
    returns the per-step results."""
    a = L.StepArgs(dt, (C.c_double * 3)(*B), 1 if first_step else 0, 1 if use_accel else 0,
                   0 if Ld is None else 1, (C.c_double * 3)(*(Ld if Ld is not None else (0.0, 0.0, 0.0))),
                   1 if inject else 0, seed, step_no, (C.c_double * 3)(*E0), 1 if efield_cg1 else 0)
    arr = _objects_in(objects)
    res = (L.StepResult * max(1, n_steps))()
    L.check(L.load().pg_run_steps(pop.handle, C.byref(a), arr, len(objects), n_steps, 1 if use_graph else 0, res))
    _objects_out(arr, objects)
    return list(res)[:n_steps]


def _tuning_dict(t) -> dict:
    return {"threads": t.threads, "blocks_per_sm": t.blocks_per_sm, "dep_agg": t.dep_agg,
            "sort_interval": t.sort_interval, "pass_ms": t.pass_ms, "sort_ms": t.sort_ms}


def set_tuning(pop: Population, threads=0, blocks_per_sm=0, dep_agg=0, sort_interval=0):
    L.check(L.load().pg_set_tuning(pop.handle, C.byref(L.Tuning(threads, blocks_per_sm, dep_agg, sort_interval))))


def get_tuning(pop: Population) -> dict:
    t = L.Tuning()
    L.check(L.load().pg_get_tuning(pop.handle, C.byref(t)))
    return _tuning_dict(t)


def autotune(pop: Population, objects, dt: float, steps_per_trial: int = 2, B=(0.0, 0.0, 0.0), first_step=False,
             inject=False, seed=0, step_no=0, E0=(0.0, 0.0, 0.0), efield_cg1=False) -> dict:
    """Autotuner of the particle pass launch and the sort interval; runs real
    steps of the simulation (see pg_autotune) and applies its choice."""
    a = L.StepArgs(dt, (C.c_double * 3)(*B), 1 if first_step else 0, 0, 0, (C.c_double * 3)(0.0, 0.0, 0.0),
                   1 if inject else 0, seed, step_no, (C.c_double * 3)(*E0), 1 if efield_cg1 else 0)
    arr = _objects_in(objects)
    t = L.Tuning()
    L.check(L.load().pg_autotune(pop.handle, C.byref(a), arr, len(objects), steps_per_trial, C.byref(t)))
    _objects_out(arr, objects)
    return _tuning_dict(t)


def set_amg_strength(pop: Population, theta: float):
    """Rebuild the AMG preconditioner with aggregation strength threshold theta
    (pg_amg_set_strength; 0, the default, counts every coupling as strong)."""
    L.check(L.load().pg_amg_set_strength(pop.handle, float(theta)))


def amg_strength(pop: Population) -> float:
    t = C.c_double()
    L.check(L.load().pg_amg_get_strength(pop.handle, C.byref(t)))
    return t.value


def autotune_amg(pop: Population, objects, dt: float, steps_per_trial: int = 6, thetas=None, B=(0.0, 0.0, 0.0),
                 first_step=False, inject=False, seed=0, step_no=0, E0=(0.0, 0.0, 0.0), efield_cg1=False) -> dict:
    """The AMG strength threshold of least PCG time over real steps of the
    simulation (pg_autotune_amg; candidates {0, 0.01, 0.02} by default);
    applies it and returns {"amg_theta", "pcg_ms"}."""
    a = L.StepArgs(dt, (C.c_double * 3)(*B), 1 if first_step else 0, 0, 0, (C.c_double * 3)(0.0, 0.0, 0.0),
                   1 if inject else 0, seed, step_no, (C.c_double * 3)(*E0), 1 if efield_cg1 else 0)
    arr = _objects_in(objects)
    cand = np.ascontiguousarray(thetas if thetas is not None else [], np.float64)
    best, ms = C.c_double(), C.c_double()
    L.check(L.load().pg_autotune_amg(pop.handle, C.byref(a), arr, len(objects), steps_per_trial,
                                     L.dptr(cand) if len(cand) else None, len(cand), C.byref(best), C.byref(ms)))
    _objects_out(arr, objects)
    return {"amg_theta": best.value, "pcg_ms": ms.value}


def adjoint_forward(pop: Population, objects, dt: float, n_steps: int, ckpt_every: int, rho_target,
                    first_step=True, use_accel=False, E0=(0.0, 0.0, 0.0), Ld=None, step_no=0) -> float:
    """K fused steps keeping checkpoints; returns ||rho_K - rho_target||^2."""
    a = L.StepArgs(dt, (C.c_double * 3)(0.0, 0.0, 0.0), 1 if first_step else 0, 1 if use_accel else 0,
                   0 if Ld is None else 1, (C.c_double * 3)(*(Ld if Ld is not None else (0.0, 0.0, 0.0))),
                   0, 0, step_no, (C.c_double * 3)(*E0), 0)
    arr = _objects_in(objects)
    tgt = np.ascontiguousarray(rho_target, np.float64)
    loss = C.c_double()
    L.check(L.load().pg_adjoint_forward(pop.handle, C.byref(a), arr, len(objects), n_steps, ckpt_every, L.dptr(tgt),
                                        C.byref(loss)))
    return loss.value


def adjoint_backward(pop: Population, n_particles: int):
    """(grad wrt initial velocities [n][3], wrt E0 [3], wrt initial positions [n][3]), by particle id."""
    gv, gx, ge = np.zeros((n_particles, 3)), np.zeros((n_particles, 3)), np.zeros(3)
    L.check(L.load().pg_adjoint_backward(pop.handle, L.dptr(gv), n_particles, L.dptr(ge), L.dptr(gx)))
    return gv, ge, gx


def adjoint_potential_gradient(pop: Population, n_objects: int) -> np.ndarray:
    """After adjoint_backward: d loss / d (fixed potential of object k)."""
    g = np.zeros(max(1, n_objects))
    L.check(L.load().pg_adjoint_potential_gradient(pop.handle, L.dptr(g), n_objects))
    return g[:n_objects]


def stage_times(pop: Population) -> dict:
    lib = L.load()
    n = C.c_int32()
    ms = np.zeros(32)
    L.check(lib.pg_stage_times(pop.handle, L.dptr(ms), 32, C.byref(n)))
    return {lib.pg_stage_name(pop.handle, k).decode(): float(ms[k]) for k in range(n.value)}


def poisson_layout(pop: Population) -> dict:
    """Stored size of the Poisson operator and of its AMG levels."""
    lib = L.load()
    out = L.PoissonLayout()
    L.check(lib.pg_poisson_layout_get(pop.handle, C.byref(out)))
    n = out.levels
    return {"n_rows": out.n_rows, "nnz": out.nnz, "sell_entries": out.sell_entries, "precond": out.precond,
            "levels": [{"rows": out.level_rows[l], "nnz": out.level_nnz[l], "nnz_p": out.level_nnz_p[l]}
                       for l in range(n)],
            "cycle_nnz_g": out.cycle_nnz_g, "cycle_nnz_u1": out.cycle_nnz_u1, "cycle_bytes": out.cycle_bytes}


def set_profiling(pop: Population, on: bool):
    L.check(L.load().pg_set_profiling(pop.handle, 1 if on else 0))
