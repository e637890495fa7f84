"""ctypes mirror of include/dropfluid.h (the C ABI of libdropfluid.so).

Constants and struct layouts here must match the header; tests check the
struct size against the library's own ``sizeof`` via ``dob_create``'s
struct_size check.
"""
from __future__ import annotations

import ctypes as C

DOB_ABI_VERSION = 1

# dob_status
DOB_OK = 0
DOB_EINVAL = -1
DOB_ENOMEM = -2
DOB_ECUDA = -3
DOB_ENOCONVERGE = -4
DOB_ETIMEOUT = -5
DOB_ESTATE = -6
STATUS_NAMES = {
    0: "DOB_OK", -1: "DOB_EINVAL", -2: "DOB_ENOMEM", -3: "DOB_ECUDA",
    -4: "DOB_ENOCONVERGE", -5: "DOB_ETIMEOUT", -6: "DOB_ESTATE",
}

DOB_BC_REFERENCE = 0
DOB_BC_CLOSED_BOX = 1

DOB_PREC_FP32 = 0
DOB_PREC_MIXED = 1
DOB_PREC_REFERENCE_FP16 = 2

DOB_PHYS_VORT_CONF = 1
DOB_PHYS_BUOYANCY = 2
DOB_PHYS_SPONGE = 4
DOB_PHYS_NECK = 8
DOB_PHYS_SOLENOIDAL = 16
DOB_PHYS_SURFACE = 32
DOB_PHYS_REFERENCE_ALL = 63
DOB_PHYS_WAVE = 64
DOB_PHYS_LIGHTING = 128

# dob_field
FIELD_VEL_U = 0
FIELD_VEL_V = 1
FIELD_VEL_W = 2
FIELD_VEL_CENTER = 3
FIELD_CURL = 4
FIELD_PRESSURE = 5
FIELD_RHS = 6
FIELD_CONC = 7
FIELD_CONC_PRED = 8
FIELD_SPLAT_INTACT = 9
FIELD_SPLAT_LYSED = 10
FIELD_WAVE = 11
FIELD_DIVERGENCE = 12
FIELD_LIGHT = 13
FIELD_BRICKS = 14
FIELD_BRICKS_RAW = 15
# adjoint fields (closed box, FP32, dye_refine 1)
FIELD_ADJ_VEL_U = 16
FIELD_ADJ_VEL_V = 17
FIELD_ADJ_VEL_W = 18
FIELD_ADJ_VEL_U2 = 19
FIELD_ADJ_VEL_V2 = 20
FIELD_ADJ_VEL_W2 = 21
FIELD_ADJ_CENTER = 22
FIELD_ADJ_CONC = 23
FIELD_ADJ_CONC2 = 24
FIELD_ADJ_PRED = 25
FIELD_ADJ_PRESSURE = 26
FIELD_ADJ_RHS = 27
ADJ_VEL_FIELDS = (FIELD_ADJ_VEL_U, FIELD_ADJ_VEL_V, FIELD_ADJ_VEL_W)
ADJ_VEL2_FIELDS = (FIELD_ADJ_VEL_U2, FIELD_ADJ_VEL_V2, FIELD_ADJ_VEL_W2)


def field_shapes(vdims, cdims, ref):
    """Host array shape and dtype of every field id (include/dropfluid.h)."""
    nz, ny, nx = vdims
    cz, cy, cx = cdims
    import numpy as np
    v = ((nz, ny, nx), np.float32)
    c = ((cz, cy, cx), np.float32)
    return {
        FIELD_VEL_U: v, FIELD_VEL_V: v, FIELD_VEL_W: v,
        FIELD_VEL_CENTER: ((nz, ny, nx, 4), np.float32),
        FIELD_CURL: ((nz, ny, nx, 4), np.float32),
        FIELD_PRESSURE: v, FIELD_RHS: v,
        FIELD_CONC: (((cz, cy, cx, 4) if ref else (cz, cy, cx)), np.float32),
        FIELD_CONC_PRED: c,
        FIELD_SPLAT_INTACT: ((cz, cy, cx), np.uint32),
        FIELD_SPLAT_LYSED: ((cz, cy, cx), np.uint32),
        FIELD_WAVE: ((WAVE_N, WAVE_N, 4), np.float32),
        FIELD_DIVERGENCE: v,
        FIELD_LIGHT: ((nz, ny, nx, 4), np.float32),
        FIELD_BRICKS: ((nz // 4, ny // 4, nx // 4), np.float32),
        FIELD_BRICKS_RAW: ((nz // 4, ny // 4, nx // 4), np.float32),
        FIELD_ADJ_VEL_U: v, FIELD_ADJ_VEL_V: v, FIELD_ADJ_VEL_W: v,
        FIELD_ADJ_VEL_U2: v, FIELD_ADJ_VEL_V2: v, FIELD_ADJ_VEL_W2: v,
        FIELD_ADJ_CENTER: ((nz, ny, nx, 4), np.float32),
        FIELD_ADJ_CONC: c, FIELD_ADJ_CONC2: c, FIELD_ADJ_PRED: c,
        FIELD_ADJ_PRESSURE: v, FIELD_ADJ_RHS: v,
    }

# dob_stage (BloodDropEngine.ts:1855-2111 order)
STAGE_ADVECT_MAC = 0
STAGE_MAC_TO_CENTER = 1
STAGE_CURL = 2
STAGE_CASSON_FORCES = 3
STAGE_MAC_RHS = 4
STAGE_PRESSURE_SOLVE = 5
STAGE_PROJECT = 6
STAGE_CLEAR_SPLATS = 7
STAGE_PARCEL_EMIT = 8
STAGE_PARCEL_ADVECT = 9
STAGE_CONC_PREDICT = 10
STAGE_CONC_RESOLVE = 11
STAGE_COUNT = 12
STAGE_NAMES = [
    "advect_mac", "mac_to_center", "curl", "casson_forces", "mac_rhs",
    "pressure_solve", "project", "clear_splats", "parcel_emit",
    "parcel_advect", "conc_predict", "conc_resolve",
]

STEP_STATS = 1
STEP_TIMING = 2
# statistics a DOB_STEP_STATS step forms (dob_set_step_stats)
STATS_RESIDUAL = 1
STATS_PARCELS = 2
STATS_ALL = 3
STEP_NO_GRAPH = 4

WAVE_N = 512
PARCEL_FLOATS = 8  # RbcParcel: posAndMass + stretchAndLysis (particles.ts:17-20)
PARTICLE_COUNT = 393216  # common.ts:18


class DobConfig(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
        ("dye_refine", C.c_uint32),
        ("dx", C.c_float), ("dt", C.c_float),
        ("domain_min", C.c_float * 3), ("domain_max", C.c_float * 3),
        ("bc_mode", C.c_int32), ("precision_mode", C.c_int32),
        ("mg_levels", C.c_int32), ("mg_pre", C.c_int32), ("mg_post", C.c_int32),
        ("mg_coarse_sweeps", C.c_int32), ("mg_cycles", C.c_int32),
        ("mg_max_outer", C.c_int32),
        ("mg_rel_tol", C.c_double),
        ("mg_div_tol", C.c_double),
        ("casson_tau_y", C.c_float), ("casson_mu_p", C.c_float),
        ("physics_flags", C.c_int32),
        ("parcel_capacity", C.c_uint32),
        ("reference_schedule", C.c_int32),
        ("vel_damping", C.c_float),
        ("dye_sharpness", C.c_float),
        ("mg_cycles_injected", C.c_int32),
    ]

    def copy(self) -> "DobConfig":
        c = DobConfig()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(DobConfig))
        return c

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            out[name] = v
        return out


class DobStepStats(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("steps_done", C.c_int32),
        ("vcycles", C.c_int32),
        ("outer_iters", C.c_int32),
        ("rhs_l2", C.c_double),
        ("residual_l2", C.c_double),
        ("max_div", C.c_double),
        ("parcels_alive", C.c_uint32),
        ("pad", C.c_uint32),
        ("stage_ms", C.c_float * STAGE_COUNT),
    ]


def config_reference() -> DobConfig:
    """The reference's own setup (common.ts:4-20, BloodDropEngine.ts:88-98):
    96x128x96 velocity grid, 192x256x192 dye, Dirichlet free-surface top,
    4-grid V-cycle with L0 1+1 / L1-L2 2+2 / L3 6 sweeps, one cycle per step,
    393216 parcels, FP32 storage (use DOB_PREC_REFERENCE_FP16 for the
    reference's rgba16float storage)."""
    c = DobConfig()
    c.struct_size = C.sizeof(DobConfig)
    c.nx, c.ny, c.nz = 96, 128, 96
    c.dye_refine = 2
    c.dx = 0.01
    c.dt = 1.0 / 60.0
    c.domain_min[:] = [-0.48, -0.98, -0.48]
    c.domain_max[:] = [0.48, 0.30, 0.48]
    c.bc_mode = DOB_BC_REFERENCE
    c.precision_mode = DOB_PREC_FP32
    c.mg_levels = 4
    c.mg_pre = 2
    c.mg_post = 2
    c.mg_coarse_sweeps = 6
    c.mg_cycles = 1
    c.mg_max_outer = 1
    c.mg_rel_tol = 0.0
    c.mg_div_tol = 0.0
    c.casson_tau_y = 0.0
    c.casson_mu_p = 0.0
    c.physics_flags = DOB_PHYS_REFERENCE_ALL
    c.parcel_capacity = PARTICLE_COUNT
    c.reference_schedule = 1
    c.vel_damping = 1.0
    c.dye_sharpness = 1.0
    c.mg_cycles_injected = 0
    return c


DENSE_COARSE_MAX = 4096     # largest coarsest grid of the exact dense solve
DENSE_COARSE_TARGET = 2304  # the closed-box hierarchy is deepened to this


def closed_box_levels(nx: int, ny: int, nz: int):
    """(mg_levels, mg_coarse_sweeps) of the closed-box configuration: the
    hierarchy is deepened (every grid keeping even dims) until the coarsest
    grid has at most DENSE_COARSE_TARGET cells, which are solved exactly (-1:
    dense inverse; 6 RBGS sweeps when no depth gets below DENSE_COARSE_MAX
    cells)."""
    levels, coarse = 1, 6
    for L in range(2, 11):
        m = 1 << L
        if nx % m or ny % m or nz % m:
            break
        cells = (nx >> (L - 1)) * (ny >> (L - 1)) * (nz >> (L - 1))
        levels = L
        coarse = -1 if cells <= DENSE_COARSE_MAX else 6
        if cells <= DENSE_COARSE_TARGET:
            break
    return levels, coarse


def config_closed_box(nx: int, ny: int, nz: int) -> DobConfig:
    """Closed box, free-slip walls, pure-Neumann pressure; FP32; 2+2 RBGS on
    every level of a hierarchy deep enough for an exact coarsest solve
    (closed_box_levels); 4 V-cycles per step; Casson
    tau_y = 0.005, mu_p = 1e-3; dx = 1, dt = 0.02 (the synthetic drop scenes).
    In the mixed mode the defect loop stops at max |div| dt/dx <= 1e-5 (at
    most 16 outer iterations of mg_cycles V-cycles each); in FP32 the first
    two steps after an injection run mg_cycles_injected = 8 V-cycles."""
    c = DobConfig()
    c.struct_size = C.sizeof(DobConfig)
    c.nx, c.ny, c.nz = nx, ny, nz
    c.dye_refine = 1
    c.dx = 1.0
    c.dt = 0.02
    c.domain_min[:] = [0.0, 0.0, 0.0]
    c.domain_max[:] = [float(nx), float(ny), float(nz)]
    c.bc_mode = DOB_BC_CLOSED_BOX
    c.precision_mode = DOB_PREC_FP32
    c.mg_levels, c.mg_coarse_sweeps = closed_box_levels(nx, ny, nz)
    c.mg_pre = 2
    c.mg_post = 2
    c.mg_cycles = 4
    c.mg_max_outer = 16
    c.mg_rel_tol = 0.0
    c.mg_div_tol = 1e-5
    c.casson_tau_y = 0.005
    c.casson_mu_p = 1e-3
    c.physics_flags = 0
    c.parcel_capacity = 8192
    c.reference_schedule = 0
    c.vel_damping = 1.0
    c.dye_sharpness = 1.0
    # the step after a drop's injection runs twice the V-cycles (a new
    # divergent source the warm start knows nothing about)
    c.mg_cycles_injected = 2 * c.mg_cycles
    return c
