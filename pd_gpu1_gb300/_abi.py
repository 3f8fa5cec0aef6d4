"""ctypes mirror of include/pd.h: parameter/cylinder/result structs, field ids, status codes.

The library itself is loaded by :mod:`pd_gpu1_gb300._lib`; this module only holds the
data types so that host code, tests and the oracle wrapper share one definition.
"""
import ctypes as C

PD_OK = 0
PD_ERR_ARG = -1
PD_ERR_CUDA = -2
PD_ERR_STATE = -3
PD_ERR_FAMILY = -4
PD_ERR_NONFINITE = -5
PD_ERR_NOMEM = -6
PD_ERR_TIMEOUT = -7
PD_ERR_UNSUPPORTED = -8

STATUS_NAMES = {
    PD_OK: "PD_OK",
    PD_ERR_ARG: "PD_ERR_ARG",
    PD_ERR_CUDA: "PD_ERR_CUDA",
    PD_ERR_STATE: "PD_ERR_STATE",
    PD_ERR_FAMILY: "PD_ERR_FAMILY",
    PD_ERR_NONFINITE: "PD_ERR_NONFINITE",
    PD_ERR_NOMEM: "PD_ERR_NOMEM",
    PD_ERR_TIMEOUT: "PD_ERR_TIMEOUT",
    PD_ERR_UNSUPPORTED: "PD_ERR_UNSUPPORTED",
}

PD_MODEL_BOND = 1
PD_MODEL_STATE = 2
PD_MODE_STATIC = 1
PD_MODE_DYNAMIC = 2

_FIELDS = [
    "X", "Y", "Z", "UX", "UY", "UZ", "VX", "VY", "VZ", "AX", "AY", "AZ", "FX", "FY", "FZ",
    "BX", "BY", "BZ", "VHX", "VHY", "VHZ", "FOX", "FOY", "FOZ", "DMG", "M", "THETA",
    "FNCST_X", "FNCST_Y", "FNCST_Z", "NN", "ROWPTR", "NL", "IDIST", "FAC", "SCR", "W", "E",
    "FAIL",
]
FIELD = {name: k for k, name in enumerate(_FIELDS)}
# element dtype per field (numpy type string)
FIELD_DTYPE = {name: "f8" for name in _FIELDS}
FIELD_DTYPE.update({"NN": "i4", "ROWPTR": "i8", "NL": "i4", "FAIL": "i4"})
BOND_FIELDS = {"NL", "IDIST", "FAC", "SCR", "W", "E", "FAIL"}


class PDParams(C.Structure):
    """pd_params (include/pd.h); the first block mirrors device_parameter (Base.cuh:46-68)."""

    _fields_ = [
        ("pi", C.c_double),
        ("N", C.c_int32), ("MN", C.c_int32), ("N_int", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("dx", C.c_double), ("emod", C.c_double), ("dens", C.c_double), ("pratio", C.c_double),
        ("bc", C.c_double), ("delta", C.c_double), ("critical_s", C.c_double), ("vol", C.c_double),
        ("dt", C.c_double),
        ("nt", C.c_int32), ("dim", C.c_int32),
        ("mass", C.c_double), ("K", C.c_double), ("G", C.c_double),
        ("model", C.c_int32), ("mode", C.c_int32),
        ("thick", C.c_double), ("length", C.c_double), ("height", C.c_double),
        ("width", C.c_double), ("load", C.c_double),
        ("sedload", C.c_double), ("break_ymin", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}

    def copy(self):
        q = PDParams()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(PDParams))
        return q


class PDCylinder(C.Structure):
    """pd_cylinder: Cylinder_Parameter (Base.cuh:227-235) plus its state (Cylinder, :237-242)."""

    _fields_ = [
        ("rad", C.c_double), ("mass", C.c_double), ("height", C.c_double), ("v", C.c_double),
        ("x", C.c_double), ("y", C.c_double), ("z", C.c_double),
        ("vel", C.c_double * 3), ("disp", C.c_double * 3), ("acc", C.c_double * 3),
        ("force", C.c_double * 3),
    ]


class PDResult(C.Structure):
    _fields_ = [
        ("N", C.c_int64), ("N_int", C.c_int64), ("B", C.c_int64),
        ("setup_ms", C.c_double), ("loop_ms", C.c_double), ("bond_updates_per_s", C.c_double),
    ]


class PDSpecimen(C.Structure):
    """pd_specimen: one plate of a batch (size, modulus, s0, pre-crack, loading rate)."""

    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("emod", C.c_double), ("critical_s", C.c_double),
        ("crack_len", C.c_double), ("crack_theta", C.c_double), ("load_scale", C.c_double),
    ]


class PDLoadStepStats(C.Structure):
    """pd_load_step_stats: one quasi-static load increment."""

    _fields_ = [
        ("iters", C.c_int32), ("warm_used", C.c_int32), ("probes", C.c_int32), ("pad_", C.c_int32),
        ("r_plain", C.c_double), ("r_start", C.c_double),
        ("r_final", C.c_double), ("ms", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}
