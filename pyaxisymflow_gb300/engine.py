"""Fused, graph-capturable per-timestep engine for many rigid-body cases.

``RigidEnsemble`` keeps every field of every case resident on one GPU and
advances all of them with one sequence of launches per step
(include/axisym_gb300.h: axi_rigid_step_f64 / _f32): the loop body of
examples/FlowPastSphere/flow_past_sphere.py:107-188 per case, with dt, drag
and time kept on the device. Cases may differ in grid size, viscosity, body
and penalisation parameters. ``precision="f64"`` is the plain path;
``"f32"`` runs the fields and transforms in FP32 with FP64 eigendecomposition,
coordinates and drag accumulation.
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .kernels.FastDiagonalisationStokesSolver import FastDiagonalisationStokesSolver
from .kernels._spectral import tf32_split
from .kernels.smooth_Heaviside import smooth_Heaviside

ST_T, ST_DT, ST_CD, ST_STEPS, ST_UMAX, ST_COUNT, ST_STATUS, ST_FORCE = range(8)
ST_UFREE, ST_LAMDT, ST_ADV, ST_C1, ST_C2, ST_ZCM, ST_UBODY, ST_DIFF, ST_FTOTAL = range(8, 17)
ST_WORDS = 24
TILE_NR, TILE_NZ = 32, 64       # stencil tile of the engine (rows x columns)
CASE_SEDIMENTING = 1


class AxiCase(ctypes.Structure):
    """Mirror of ``axi_case`` in include/axisym_gb300.h."""
    _fields_ = [
        ("nr", ctypes.c_int32), ("nz", ctypes.c_int32), ("kill_width", ctypes.c_int32),
        ("stencil_tile0", ctypes.c_int32),
        ("dx", ctypes.c_double), ("nu", ctypes.c_double), ("lam", ctypes.c_double),
        ("U0", ctypes.c_double), ("t_ramp", ctypes.c_double), ("cfl", ctypes.c_double),
        ("U_body", ctypes.c_double), ("cd_scale", ctypes.c_double),
        ("dt_diff", ctypes.c_double), ("eps", ctypes.c_double),
        ("inv_dx2", ctypes.c_double), ("inv_2dx", ctypes.c_double),
        ("flags", ctypes.c_int32), ("pad0", ctypes.c_int32),
        ("rho_f", ctypes.c_double), ("rho_s", ctypes.c_double), ("grav", ctypes.c_double),
        ("part_mass", ctypes.c_double), ("part_vol", ctypes.c_double),
        ("r_body", ctypes.c_double), ("blend_w", ctypes.c_double),
        ("omega", ctypes.c_void_p), ("psi", ctypes.c_void_p), ("u_z", ctypes.c_void_p),
        ("u_r", ctypes.c_void_p), ("chi", ctypes.c_void_p), ("kill_coef", ctypes.c_void_p),
        ("r", ctypes.c_void_p), ("z", ctypes.c_void_p), ("rinv2dx", ctypes.c_void_p),
        ("rinv2", ctypes.c_void_p), ("rw", ctypes.c_void_p), ("zw", ctypes.c_void_p),
        ("Er", ctypes.c_void_p), ("Er_inv_w", ctypes.c_void_p), ("EzinvT", ctypes.c_void_p),
        ("EzT", ctypes.c_void_p), ("inv_eig", ctypes.c_void_p),
        ("gemm_work", ctypes.c_void_p), ("state", ctypes.c_void_p),
        ("partials", ctypes.c_void_p), ("history", ctypes.c_void_p),
        ("history_len", ctypes.c_int64),
        ("omega_hi", ctypes.c_void_p), ("omega_lo", ctypes.c_void_p),
        ("tc_basis", ctypes.c_void_p * 8), ("tc_work", ctypes.c_void_p * 4),
        ("dct_table", ctypes.c_void_p),
        ("psi_lo", ctypes.c_void_p),
    ]




@dataclass
class RigidBodyCase:
    """One flow-past-a-rigid-body case (defaults: the 512 x 256 sphere,
    z in [0, 2], r in [0, 1], Re 100)."""
    nz: int = 512
    nr: int = 256
    dx: float = 1.0 / 256
    z_cm: float = 0.5
    r_sphere: float = 0.0625
    U0: float = 1.0
    Re: float = 100.0
    lam: float = 1e4
    cfl: float = 0.1
    kill_width: int = 3
    ramp: bool = True
    noise: float = 1e-6
    seed: int = 0
    body: str = "sphere"       # sphere | spheroid | torus
    aspect: float = 1.0        # spheroid: axial / radial semi-axis
    torus_R: float = 0.0       # torus: ring radius (r_sphere is the tube radius)
    U_body: float = 0.0
    # freely sedimenting sphere (examples/SedimentingRigidSphere/falling_rigid_sphere.py):
    # no free stream, body velocity / position integrated on the device
    sediment: bool = False
    rho_f: float = 1.0
    rho_s: float = 1.1
    gravity: float = 9.81
    U_ref: float = 1.0         # velocity scale of Re when U0 = 0

    @property
    def nu(self):
        u = self.U0 if self.U0 != 0 else self.U_ref
        return u * 2 * self.r_sphere / self.Re

    @property
    def t_ramp(self):
        return 20 * self.r_sphere / self.U0 if self.U0 != 0 else 0.0

    @property
    def moll_zone(self):
        return self.dx * 2 ** 0.5

    def level_set(self, Z, R):
        """Signed distance-like level set, positive inside the body
        (examples/FlowPastSphere/flow_past_sphere.py:81,
        examples/SpheroidStreaming/spheroid_streaming.py:92-96,
        examples/TorusStreaming/torus_streaming.py:94-96)."""
        if self.body == "sphere":
            return -np.sqrt((Z - self.z_cm) ** 2 + R ** 2) + self.r_sphere
        if self.body == "spheroid":
            a, b = self.r_sphere * self.aspect, self.r_sphere
            return self.r_sphere * (1.0 - np.sqrt(((Z - self.z_cm) / a) ** 2 + (R / b) ** 2))
        if self.body == "torus":
            return -np.sqrt((Z - self.z_cm) ** 2 + (R - self.torus_R) ** 2) + self.r_sphere
        raise ValueError(f"unknown body {self.body!r}")


def grid(nz, nr, dx):
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    return z, r


def kill_coefficients(z, r, width, dx):
    """Sine-taper factors of kernels/kill_boundary_vorticity_sine.py:9-26, with
    the reference's own expression (literal 1 - Z, 1 - R): z start, z end,
    outer r, each `width` long."""
    zs = np.sin(np.pi * (z[:width] - 0.5 * dx) / 2 / (width - 1) / dx)
    ze = np.sin(np.pi * (1 - z[-width:] - 0.5 * dx) / 2 / (width - 1) / dx)
    rr = np.sin(np.pi * (1 - r[-width:] - 0.5 * dx) / 2 / (width - 1) / dx)
    return np.concatenate([zs, ze, rr])


class AxiTuning(ctypes.Structure):
    """Mirror of ``axi_tuning`` in include/axisym_gb300.h: launch choices that
    change scheduling only (bit-identical results); 0 = default."""
    _fields_ = [("stencil_blocks_per_sm", ctypes.c_int32 * 3),
                ("prefetch_waves", ctypes.c_int32), ("tc_ctas_percent", ctypes.c_int32),
                ("tc_tile_order", ctypes.c_int32), ("dct_item_order", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


# names of the launch choices (keys of RigidEnsemble.tuning); plan_groups is
# the host's (how many plans the cases are split into, each stepped on a
# stream of its own: 0 automatic, see RigidEnsemble.plan_group_count), the
# others go to the plan (axi_tuning)
TUNING_KEYS = ("vel_max_blocks", "penalise_blocks", "advect_blocks", "prefetch_waves",
               "tc_ctas_percent", "tc_tile_order", "dct_item_order", "plan_groups")


def fill_tuning(tune, choices):
    """Writes a dict of launch choices (TUNING_KEYS) into an AxiTuning."""
    unknown = set(choices) - set(TUNING_KEYS)
    if unknown:
        raise ValueError(f"unknown launch choices {sorted(unknown)}")
    for q, k in enumerate(("vel_max_blocks", "penalise_blocks", "advect_blocks")):
        tune.stencil_blocks_per_sm[q] = int(choices.get(k, 0))
    for k in ("prefetch_waves", "tc_ctas_percent", "tc_tile_order", "dct_item_order"):
        setattr(tune, k, int(choices.get(k, 0)))


class AxiPlanInfo(ctypes.Structure):
    """Mirror of ``axi_plan_info`` in include/axisym_gb300.h."""
    _fields_ = [("n_cases", ctypes.c_int32), ("n_stencil_tiles", ctypes.c_int32),
                ("n_gemm_tiles", ctypes.c_int32), ("elem_bytes", ctypes.c_int32),
                ("bytes", ctypes.c_int64), ("flags", ctypes.c_int32),
                ("n_tc_tiles", ctypes.c_int32 * 4), ("n_dct_items", ctypes.c_int32),
                ("tune", AxiTuning)]


PLAN_TENSOR_CORES = 1
PLAN_DCT_Z = 2
PLAN_REFINE = 4


def dct_ok(nz, precision="f32"):
    """nz the z transform handles as a DCT: even, factors 2 and 3 only, at most
    4096 (float engine) or 2048 (double engine)."""
    n = int(nz)
    if n < 2 or n % 2 or n > (4096 if precision == "f32" else 2048):
        return False
    for f in (2, 3):
        while n % f == 0:
            n //= f
    return n == 1


def dct_table(nz, dtype=np.float32):
    """Tables of the z transform (layout of axi_case.dct_table), float for the
    float engine, double for the double engine: exp(-2 pi i m / nz) as
    (cos, sin), (cos, sin)(pi k / 2 nz), c_k, 1 / c_k."""
    m = np.arange(nz, dtype=np.float64)
    tw = np.stack([np.cos(2 * np.pi * m / nz), -np.sin(2 * np.pi * m / nz)], axis=1)
    rot = np.stack([np.cos(np.pi * m / (2 * nz)), np.sin(np.pi * m / (2 * nz))], axis=1)
    c = np.full(nz, np.sqrt(2.0 / nz))
    c[0] = np.sqrt(1.0 / nz)
    return np.concatenate([tw.ravel(), rot.ravel(), c, 1.0 / c]).astype(dtype)


class _Bases:
    """Spectral bases shared by all cases with the same (nr, nz, dx).

    With `dct`, the z eigenbasis is the orthonormal DCT-II basis (the Neumann
    z operator of the solver is diagonal in it): the z products become
    transforms, inv_eig is 1 / (lambda_r_i + lambda_z_k) in DCT order and only
    the radial operands are kept for the tensor cores."""

    def __init__(self, nr, nz, dx, dtype, device, tensor_cores=False, dct=False):
        solver = FastDiagonalisationStokesSolver(nr, nz, dx, device=device)
        d = solver.engine.dev
        self.t = {k: d[k].to(dtype).contiguous() for k in
                  ("Er", "Er_inv_w", "EzinvT", "EzT", "inv_eig")}
        self.tc = []
        self.dct_table = None
        if dct:
            lam_z = (2.0 - 2.0 * np.cos(np.pi * np.arange(nz) / nz)) / (dx * dx)
            inv = 1.0 / (solver.engine.eig_vals_r.reshape(nr, 1) + lam_z.reshape(1, nz))
            self.t["inv_eig"] = torch.tensor(inv, dtype=dtype, device=device)
            self.dct_table = torch.tensor(
                dct_table(nz, np.float64 if dtype == torch.float64 else np.float32), device=device)
        if tensor_cores:
            h = solver.engine.host
            # operands of the K-major tensor-core form (C = A B^T per stage):
            # E_z^-1, E_r^-1 diag(r), E_z, E_r (the z ones unused with dct)
            for k, m in enumerate((h["EzinvT"].T, h["Er_inv_w"], h["EzT"].T, h["Er"])):
                if dct and k in (0, 2):
                    self.tc += [None, None]
                    continue
                hi, lo = tf32_split(np.ascontiguousarray(m))
                self.tc.append(torch.tensor(hi, device=device))
                self.tc.append(torch.tensor(lo, device=device))


class CaseState:
    """Device-resident fields and per-case state of one case of an ensemble.

    It survives re-planning, so cases can join and leave an ensemble between
    steps (continuous batching) without disturbing the others."""

    def __init__(self, ens, case, slot, history_steps=0, initial_vorticity=None):
        self.case = c = case
        self.slot = slot
        dev = ens.device
        dtype = ens.dtype
        f = dict(dtype=dtype, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        z, r = grid(c.nz, c.nr, c.dx)
        Z, R = np.meshgrid(z, r)
        b = ens._bases_for(c)
        self.bases = b
        if initial_vorticity is not None:
            w0 = np.asarray(initial_vorticity, dtype=np.float64)
        else:
            w0 = c.noise * np.random.default_rng(c.seed).standard_normal((c.nr, c.nz))
        chi64 = torch.zeros((c.nr, c.nz), **f64)
        smooth_Heaviside(chi64, torch.tensor(c.level_set(Z, R), **f64), c.moll_zone)
        t = dict(
            omega=torch.tensor(w0, **f64).to(dtype),
            psi=torch.zeros((c.nr, c.nz), **f),
            u_z=torch.zeros((c.nr, c.nz), **f),
            u_r=torch.zeros((c.nr, c.nz), **f),
            chi=chi64.to(dtype),
            kill_coef=torch.tensor(kill_coefficients(z, r, c.kill_width, c.dx), **f64),
            r=torch.tensor(r, **f64),
            z=torch.tensor(z, **f64),
            rinv2dx=torch.tensor(1.0 / (2 * c.dx * r), **f64).to(dtype),
            rinv2=torch.tensor(1.0 / (r * r), **f64).to(dtype),
            rw=torch.tensor(r, **f64).to(dtype),
            zw=torch.tensor(z, **f64).to(dtype),
            gemm_work=torch.zeros(2 * c.nr * c.nz, **f),
            partials=torch.zeros(2 * ((c.nr + TILE_NR - 1) // TILE_NR)
                                 * ((c.nz + TILE_NZ - 1) // TILE_NZ) + 8, **f64),
        )
        if ens.tensor_cores and not ens.dct:
            # the operand pair describes the stored float32 field, exactly as
            # the device refresh (axi_rigid_refresh_operands) computes it
            whi, wlo = tf32_split(np.asarray(w0, dtype=np.float32))
            t["omega_hi"] = torch.tensor(whi, device=dev)
            t["omega_lo"] = torch.tensor(wlo, device=dev)
        if ens.tensor_cores:
            t["tc_work"] = [torch.zeros(c.nr * c.nz, dtype=torch.float32, device=dev)
                            for _ in range(4)]
        if ens.refine:
            # low part of psi: the refined solve keeps psi as psi + psi_lo
            t["psi_lo"] = torch.zeros((c.nr, c.nz), dtype=torch.float32, device=dev)
        self.fields = t
        self.history = (torch.zeros((history_steps, 2), **f64) if history_steps else None)
        st = ens.state_arena[slot]
        st.zero_()
        s = AxiCase()
        s.nr, s.nz, s.kill_width = c.nr, c.nz, c.kill_width
        s.dx, s.nu, s.lam, s.U0 = c.dx, c.nu, c.lam, c.U0
        s.t_ramp = c.t_ramp if c.ramp else 0.0
        s.cfl, s.U_body = c.cfl, c.U_body
        s.cd_scale = 2 * 2 * math.pi * c.dx * c.dx * c.lam / (math.pi * c.r_sphere ** 2)
        s.dt_diff = 0.9 * c.dx ** 2 / 4 / c.nu
        s.eps = float(np.finfo(float).eps)
        s.inv_dx2 = 1.0 / (c.dx * c.dx)
        s.inv_2dx = 0.5 / c.dx
        if c.sediment:
            if c.body != "sphere":
                raise ValueError("sedimenting bodies are spheres")
            # falling_rigid_sphere.py:71-73 (mass and volume from the initial mask)
            chi_h = chi64.cpu().numpy()
            s.flags = CASE_SEDIMENTING
            s.rho_f, s.rho_s = c.rho_f, c.rho_s
            s.grav = (c.rho_s - c.rho_f) * c.gravity
            s.part_mass = 2 * np.pi * c.dx * c.dx * c.rho_s * np.sum(chi_h * R)
            s.part_vol = 2 * np.pi * c.dx * c.dx * np.sum(chi_h * R)
            s.r_body = c.r_sphere
            s.blend_w = c.moll_zone
            st[ST_ZCM] = c.z_cm
        for name in ("omega", "psi", "u_z", "u_r", "chi", "kill_coef", "r", "z",
                     "rinv2dx", "rinv2", "rw", "zw", "gemm_work", "partials"):
            setattr(s, name, t[name].data_ptr())
        for name, v in b.t.items():
            setattr(s, name, v.data_ptr())
        if ens.tensor_cores:
            if not ens.dct:
                s.omega_hi = t["omega_hi"].data_ptr()
                s.omega_lo = t["omega_lo"].data_ptr()
            for q in range(8):
                s.tc_basis[q] = b.tc[q].data_ptr() if b.tc[q] is not None else None
            for q in range(4):
                s.tc_work[q] = t["tc_work"][q].data_ptr()
        if ens.dct:
            s.dct_table = b.dct_table.data_ptr()
        if ens.refine:
            s.psi_lo = t["psi_lo"].data_ptr()
        s.state = st.data_ptr()
        if self.history is not None:
            s.history = self.history.data_ptr()
            s.history_len = history_steps
        self.struct = s

    def nbytes(self):
        n = 0
        for v in self.fields.values():
            for x in (v if isinstance(v, list) else [v]):
                n += x.numel() * x.element_size()
        return n


def split_by_cells(cases, groups):
    """Indices of `cases` in `groups` parts of about equal cell count (greedy,
    largest case first), each part in input order; empty parts dropped."""
    groups = max(1, min(groups, len(cases)))
    order = sorted(range(len(cases)), key=lambda k: -cases[k].nr * cases[k].nz)
    load = [0] * groups
    parts = [[] for _ in range(groups)]
    for k in order:
        g = load.index(min(load))
        parts[g].append(k)
        load[g] += cases[k].nr * cases[k].nz
    return [sorted(p) for p in parts if p]


class RigidEnsemble:
    """Cases resident on one GPU, advanced together by one launch sequence per
    step. Cases may join (add_case) and leave (remove_case) between steps.

    The cases may be split into plan groups (launch choice plan_groups), each
    with a plan of its own; a step then forks one stream per group from the
    caller's stream and joins them again, so the kernels of one group fill
    the other's drain and fill bubbles between kernels (the 64-case bench
    workload: 0.808 ms per step as one plan, 0.769 ms as two, 0.788 as
    three). Each case's arithmetic does not depend on the grouping."""

    # plan groups of the automatic choice, and the fewest cases it splits
    AUTO_PLAN_GROUPS = 2
    AUTO_SPLIT_MIN_CASES = 8

    def __init__(self, cases, precision="f64", device="cuda", history_steps=0,
                 initial_vorticity=None, tensor_cores=None, capacity=None, dct=None,
                 refine=None):
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        if tensor_cores is None:
            tensor_cores = precision == "f32"
        if tensor_cores and precision != "f32":
            raise ValueError("tensor-core products are for the f32 engine")
        cases = list(cases)
        if dct is None:
            # z products as DCTs when every case's nz allows it (faster than
            # the dense z products: tensor-core ones in the float engine, SIMT
            # FP64 ones in the double engine); the float engine's DCT feeds
            # the tensor-core radial products only
            dct = ((tensor_cores or precision == "f64")
                   and all(dct_ok(c.nz, precision) for c in cases))
        if dct and precision == "f32" and not tensor_cores:
            raise ValueError("the float DCT z transform goes with the tensor-core products")
        if refine is None:
            # each solve one refinement step from the psi of the previous step
            refine = dct and precision == "f32"
        if refine and (not dct or precision != "f32"):
            raise ValueError("refinement of the solve runs in the float engine with the DCT "
                             "z transform")
        self.tensor_cores = tensor_cores
        self.dct = dct
        self.refine = refine
        self.precision = precision
        self.dtype = torch.float64 if precision == "f64" else torch.float32
        self.device = torch.device(device)
        capacity = max(capacity or 0, len(cases), 1)
        self.state_arena = torch.zeros((capacity, ST_WORDS), dtype=torch.float64,
                                       device=self.device)
        self._free = list(range(capacity - 1, -1, -1))
        self._bases = {}
        self.members = []
        self._omega_arena = None
        self.graph = None
        self.tuning = {}
        self.plans = []
        self._streams = []
        lib = N.lib()
        self._step_fn = getattr(lib, f"axi_rigid_step_{precision}")
        self._phase_fn = getattr(lib, f"axi_rigid_phase_{precision}")
        for k, c in enumerate(cases):
            w0 = initial_vorticity[k] if initial_vorticity is not None else None
            self._admit(c, history_steps, w0)
        self._replan()

    def _bases_for(self, c):
        key = (c.nr, c.nz, c.dx)
        if key not in self._bases:
            self._bases[key] = _Bases(c.nr, c.nz, c.dx, self.dtype, self.device,
                                      tensor_cores=self.tensor_cores, dct=self.dct)
        return self._bases[key]

    def _admit(self, case, history_steps=0, initial_vorticity=None):
        if not self._free:
            raise RuntimeError("ensemble is at capacity")
        if self.dct and not dct_ok(case.nz, self.precision):
            raise ValueError(f"nz = {case.nz} has no DCT plan (even, factors 2 and 3 only); "
                             "build the ensemble with dct=False for such grids")
        m = CaseState(self, case, self._free.pop(), history_steps, initial_vorticity)
        self.members.append(m)
        return m

    @property
    def omega_arena(self):
        """Every member's omega in one contiguous device buffer (members in
        order, each (nr, nz) row-major); a plan made without packing is made
        again with it on first use."""
        if self._omega_arena is None and self.members:
            self._replan(pack=True)
        return self._omega_arena

    def _pack_vorticity(self):
        """Place every member's omega in one contiguous device arena, so host
        transfers of all cases' vorticity are one copy each way."""
        n = sum(m.case.nr * m.case.nz for m in self.members)
        arena = torch.empty(max(n, 1), dtype=self.dtype, device=self.device)
        off = 0
        for m in self.members:
            c = m.case
            view = arena[off:off + c.nr * c.nz].view(c.nr, c.nz)
            view.copy_(m.fields["omega"])
            m.fields["omega"] = view
            m.struct.omega = view.data_ptr()
            off += c.nr * c.nz
        self._omega_arena = arena[:n]

    def _replan(self, pack=True):
        """Rebuild and upload the plan for the current members. pack=False
        leaves each omega where it is (no copy of every case's vorticity; the
        continuous-batching server re-plans at every admission and
        retirement and never needs the arena)."""
        self.graph = None
        n = len(self.members)
        if pack:
            self._pack_vorticity()
        else:
            self._omega_arena = None
        self.plans = []
        self.info = AxiPlanInfo()
        fill_tuning(self.info.tune, self.tuning)
        if n == 0:
            self.plan = None
            self.n_tiles = 0
            return
        lib = N.lib()
        esize = 8 if self.precision == "f64" else 4
        flags = ((PLAN_TENSOR_CORES if self.tensor_cores else 0) | (PLAN_DCT_Z if self.dct else 0)
                 | (PLAN_REFINE if self.refine else 0))
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        for idx in split_by_cells(self.cases, self.plan_group_count(n)):
            structs = (AxiCase * len(idx))()
            for q, k in enumerate(idx):
                structs[q] = self.members[k].struct
            info = AxiPlanInfo()
            fill_tuning(info.tune, self.tuning)
            N.check(lib.axi_plan_init(ctypes.addressof(structs), len(idx), esize, flags,
                                      ctypes.byref(info)), "plan_init")
            plan = torch.empty(int(info.bytes), dtype=torch.uint8, device=self.device)
            N.check(lib.axi_plan_upload(ctypes.addressof(structs), ctypes.byref(info),
                                        ctypes.c_void_p(plan.data_ptr()), stream), "plan_upload")
            self.plans.append((info, plan, structs, idx))
        self.info, self.plan = self.plans[0][0], self.plans[0][1]
        self.n_tiles = sum(p[0].n_stencil_tiles for p in self.plans)

    def plan_group_count(self, n=None):
        """Plan groups for n cases (default: the members): the plan_groups
        launch choice, or when it is 0 (automatic) AUTO_PLAN_GROUPS once there
        are AUTO_SPLIT_MIN_CASES cases, else one."""
        n = len(self.members) if n is None else n
        g = int(self.tuning.get("plan_groups", 0))
        if g <= 0:
            g = self.AUTO_PLAN_GROUPS if n >= self.AUTO_SPLIT_MIN_CASES else 1
        return max(1, min(g, n))

    @property
    def n_plans(self):
        return len(self.plans)

    def _group_streams(self):
        while len(self._streams) < len(self.plans):
            self._streams.append(torch.cuda.Stream(self.device))
        return self._streams[:len(self.plans)]

    def set_tuning(self, choices):
        """Use the launch choices `choices` (a dict over TUNING_KEYS; missing
        keys take the default) from the next step on. They change how the
        work is scheduled, never the results. Re-plans (a captured graph must
        be captured again)."""
        fill_tuning(AxiTuning(), choices)  # validates the keys
        self.tuning = dict(choices)
        self._replan()

    def add_case(self, case, history_steps=0, initial_vorticity=None):
        """Admit a case between steps; returns its CaseState."""
        m = self._admit(case, history_steps, initial_vorticity)
        self._replan()
        return m

    def remove_case(self, member):
        """Retire a case between steps (its device memory is released)."""
        self.members.remove(member)
        self._free.append(member.slot)
        member.fields = None
        self._replan()

    @property
    def cases(self):
        return [m.case for m in self.members]

    @property
    def fields(self):
        return [m.fields for m in self.members]

    @property
    def history(self):
        if not self.members or self.members[0].history is None:
            return None
        return torch.stack([m.history for m in self.members])

    @property
    def state(self):
        idx = [m.slot for m in self.members]
        if idx == list(range(len(idx))):
            return self.state_arena[:len(idx)]
        return self.state_arena[idx]

    @property
    def n_cases(self):
        return len(self.members)

    def cells(self):
        return sum(c.nr * c.nz for c in self.cases)

    def _forked(self, fn, arg, what, stream):
        """fn(info, plan, arg, stream) for every plan group: on `stream` for
        one group, else on streams forked from it and joined back."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        if len(self.plans) == 1:
            N.check(fn(ctypes.byref(self.info), ctypes.c_void_p(self.plan.data_ptr()), int(arg),
                       ctypes.c_void_p(s.cuda_stream)), what)
            return
        streams = self._group_streams()
        for (info, plan, _, _), gs in zip(self.plans, streams):
            gs.wait_stream(s)
            N.check(fn(ctypes.byref(info), ctypes.c_void_p(plan.data_ptr()), int(arg),
                       ctypes.c_void_p(gs.cuda_stream)), what)
        for gs in streams:
            s.wait_stream(gs)

    def step(self, n=1, stream=None):
        """Advance every case by n steps (asynchronous on torch's current
        stream, or `stream`). With several plan groups each group's steps run
        on a stream forked from it and joined back before the call returns."""
        self._forked(self._step_fn, n, "rigid_step", stream)

    PHASES = ("kill", "transform", "vel_max", "penalise", "advect_diffuse")
    # the four launches of "transform" (phase ids 5..8), for timing
    TRANSFORM_PARTS = ("z_forward", "r_product", "z_inverse", "r_product_2")

    def phase(self, ph, stream=None):
        """Run one phase of a step (see PHASES); all six in order = one step.
        The plan groups run it concurrently, as in a step (forked streams)."""
        self._forked(self._phase_fn, ph, "rigid_phase", stream)

    def capture(self, steps_per_replay=1):
        """Capture `steps_per_replay` steps into a CUDA graph (replay with replay())."""
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(steps_per_replay, stream=s)
        torch.cuda.synchronize(self.device)
        self.graph = g
        self.graph_steps = steps_per_replay
        return g

    def replay(self):
        self.graph.replay()

    def status(self):
        """Sticky status bits per case (0 = healthy); a failed asynchronous copy
        (tensor-core products or stencil boxes) marks every case with bit
        1 << AXI_ERR_CUDA."""
        st = self.state[:, ST_STATUS].cpu().numpy().view(np.uint64)
        out = (st & 0xFFFFFFFF).astype(np.int64)
        for info, plan, _, _ in self.plans:
            err = ctypes.c_int(0)
            N.check(N.lib().axi_plan_tc_status(
                ctypes.byref(info), ctypes.c_void_p(plan.data_ptr()),
                ctypes.byref(err), ctypes.c_void_p(
                    torch.cuda.current_stream(self.device).cuda_stream)), "plan_tc_status")
            if err.value:
                out |= 1 << N.AXI_ERR_CUDA
        return out

    def refresh_operands(self, stream=None):
        """After writing omega of any case directly, recompute the tensor-core
        operand copy of omega (one launch for all cases)."""
        if self.tensor_cores:
            s = stream if stream is not None else torch.cuda.current_stream(self.device)
            for info, plan, _, _ in self.plans:
                N.check(N.lib().axi_rigid_refresh_operands(
                    ctypes.byref(info), ctypes.c_void_p(plan.data_ptr()),
                    ctypes.c_void_p(s.cuda_stream)), "rigid_refresh_operands")

    def load_vorticity(self, src, stream=None):
        """Replace the vorticity of every case from one flat buffer laid out like
        omega_arena (e.g. pinned host memory): one copy, then the tensor-core
        operand refresh. Asynchronous on the stream."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            self.omega_arena.copy_(src.view(-1), non_blocking=True)
        self.refresh_operands(stream=s)

    def store_vorticity(self, dst, stream=None):
        """Copy the vorticity of every case into one flat buffer laid out like
        omega_arena (one copy; asynchronous on the stream)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            dst.view(-1).copy_(self.omega_arena, non_blocking=True)

    def set_vorticity(self, k, w):
        """Replace the vorticity of case k (keeps the tensor-core operand copy in step)."""
        self.fields[k]["omega"].copy_(w)
        self.refresh_operands()

    def vorticity(self, k):
        return self.fields[k]["omega"]

    def time(self):
        return self.state[:, ST_T].cpu().numpy()


class HostPipeline:
    """Cases whose vorticity lives in host memory, advanced one step per call
    with the host transfers overlapped with computation.

    The cases are split into `groups` sub-ensembles of about equal size, each
    with its own stream. One step() issues, per group: the H2D copy of the
    group's vorticity (load_vorticity), one step, and the D2H copy back
    (store_vorticity). Groups run concurrently, so while one group computes
    the copy engines move the next group's input and the previous group's
    output; with capture_pipelined the steps themselves overlap as well (on
    the 64-case workload, each group one plan: 2.09e10 cell-updates/s with
    two groups, 2.03e10 with four, 1.87e10 with eight). Every case's result
    is the same as in a single RigidEnsemble.
    """

    def __init__(self, cases, groups=2, precision="f32", device="cuda", **kw):
        cases = list(cases)
        # greedy balance by cells, keeping each group's cases in input order
        self.index = split_by_cells(cases, groups)
        self.device = torch.device(device)
        self.ensembles = [RigidEnsemble([cases[k] for k in idx], precision=precision,
                                        device=self.device, **kw) for idx in self.index]
        self.streams = [torch.cuda.Stream(self.device) for _ in self.ensembles]
        self.graph = None
        self.dtype = self.ensembles[0].dtype
        # one flat host buffer: the groups' arenas back to back
        self.offsets = [0]
        for e in self.ensembles:
            self.offsets.append(self.offsets[-1] + e.omega_arena.numel())

    def cells(self):
        return sum(e.cells() for e in self.ensembles)

    def host_buffer(self):
        """A pinned host buffer holding every case's vorticity (group arenas
        back to back), filled with the current device values."""
        h = torch.empty(self.offsets[-1], dtype=self.dtype, pin_memory=True)
        for e, a, b in zip(self.ensembles, self.offsets, self.offsets[1:]):
            h[a:b].copy_(e.omega_arena)
        return h

    def _group_step(self, g, host, state_out, s):
        """Group g's step on stream s: its vorticity in, one step, vorticity
        and state blocks out."""
        e = self.ensembles[g]
        a, b = self.offsets[g], self.offsets[g + 1]
        with torch.cuda.stream(s):
            e.load_vorticity(host[a:b], stream=s)
            e.step(1, stream=s)
            e.store_vorticity(host[a:b], stream=s)
            if state_out is not None:
                row = sum(len(idx) for idx in self.index[:g])
                state_out[row:row + e.n_cases].copy_(e.state, non_blocking=True)

    def step(self, host, state_out=None):
        """One step of every case: host vorticity in, step, host vorticity out.
        Asynchronous; call synchronize() before reading `host`. state_out
        (pinned, one row of AXI_ST_WORDS per case, groups in order) receives
        each case's state block."""
        cur = torch.cuda.current_stream(self.device)
        for g, s in enumerate(self.streams):
            s.wait_stream(cur)
            self._group_step(g, host, state_out, s)
        for s in self.streams:
            cur.wait_stream(s)

    def capture(self, host, state_out=None):
        """Record step(host, state_out) as one CUDA graph; replay() then issues
        every group's copies and launches at once (about 0.1 ms of host work
        per group saved each step). The graph holds the buffers' addresses:
        host and state_out must stay alive and in place while it is used."""
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(host, state_out)
        torch.cuda.synchronize(self.device)
        self.graph = g
        self._graph_buffers = (host, state_out)
        return g

    def replay(self):
        """One captured step (asynchronous on the current stream)."""
        self.graph.replay()

    def capture_pipelined(self, host, state_outs):
        """Record each group's step as a CUDA graph of its own, once per host
        state buffer in `state_outs` (steps take the buffers in turn), for
        replay_step / wait_step. A group's step then follows only its own
        previous step on its stream: while the last groups of step k still
        compute, the first groups already copy in and advance step k + 1, so
        the copies and the steps of successive steps overlap. The graphs hold
        the buffers' addresses: host and state_outs must stay alive and in
        place while they are used."""
        torch.cuda.synchronize(self.device)
        graphs = []
        for st in state_outs:
            row = []
            for g, s in enumerate(self.streams):
                gr = torch.cuda.CUDAGraph()
                with torch.cuda.stream(s):
                    with torch.cuda.graph(gr, stream=s):
                        self._group_step(g, host, st, s)
                row.append(gr)
            graphs.append(row)
        torch.cuda.synchronize(self.device)
        self.step_graphs = graphs
        self.step_done = [[torch.cuda.Event() for _ in self.streams] for _ in state_outs]
        self._pipelined_buffers = (host, list(state_outs))

    def replay_step(self, k):
        """Issue step k (asynchronous): every group's graph on its own stream.
        Its state blocks go to state_outs[k % len(state_outs)]; before step
        k + len(state_outs) is issued, wait_step(k) must have returned and the
        caller must be done reading that buffer."""
        p = k % len(self.step_graphs)
        for gr, s, ev in zip(self.step_graphs[p], self.streams, self.step_done[p]):
            with torch.cuda.stream(s):
                gr.replay()
                ev.record(s)
        return p

    def wait_step(self, k):
        """Block until step k's copies to the host are complete; returns the
        index of the state buffer that holds its state blocks."""
        p = k % len(self.step_graphs)
        for ev in self.step_done[p]:
            ev.synchronize()
        return p

    def synchronize(self):
        for s in self.streams:
            s.synchronize()
        torch.cuda.current_stream(self.device).synchronize()

