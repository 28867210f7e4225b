"""ctypes mirror of ``parrsb_options`` (include/parrsb.h).

The layout is byte-identical to the reference's option struct
(src/parRSB.h:21-41): fourteen ``int`` fields and one ``double`` in this
order.  Defaults follow src/parrsb.c:26-44.
"""
import ctypes

FIELDS = [
    ("partitioner", ctypes.c_int),
    ("tagged", ctypes.c_int),
    ("levels", ctypes.c_int),
    ("find_disconnected_comps", ctypes.c_int),
    ("repair", ctypes.c_int),
    ("verbose_level", ctypes.c_int),
    ("profile_level", ctypes.c_int),
    ("rsb_algo", ctypes.c_int),
    ("rsb_pre", ctypes.c_int),
    ("rsb_max_iter", ctypes.c_int),
    ("rsb_max_passes", ctypes.c_int),
    ("rsb_tol", ctypes.c_double),
    ("rsb_dump_stats", ctypes.c_int),
    ("rsb_mg_grammian", ctypes.c_int),
    ("rsb_mg_factor", ctypes.c_int),
]

DEFAULTS = dict(
    partitioner=0, tagged=0, levels=2, find_disconnected_comps=1, repair=0,
    verbose_level=1, profile_level=0, rsb_algo=0, rsb_pre=1, rsb_max_iter=50,
    rsb_max_passes=50, rsb_tol=1e-5, rsb_dump_stats=0, rsb_mg_grammian=0,
    rsb_mg_factor=2)


class ParrsbOptions(ctypes.Structure):
    _fields_ = FIELDS

    @classmethod
    def make(cls, **kw):
        vals = dict(DEFAULTS)
        for k in kw:
            if k not in vals:
                raise KeyError(f"unknown parrsb option {k!r}")
        vals.update(kw)
        return cls(**vals)

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in FIELDS}


# Return codes of include/parrsb.h
OK, ERR_ARGS, ERR_CUDA, ERR_CHECK, ERR_UNSUPPORTED = 0, 1, 2, 3, 4
