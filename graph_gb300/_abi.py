"""ctypes mirror of include/cgl.h (structs, status codes, stage bits)."""
import ctypes as C
import math

CGL_OK = 0
CGL_INVALID_ARG = 1
CGL_OOM = 2
CGL_CUDA_ERROR = 3
CGL_DEVICE_TIMEOUT = 4
CGL_DESTROYED = 5
CGL_WARNING = 6

STATUS_NAMES = {
    CGL_OK: "OK", CGL_INVALID_ARG: "INVALID_ARG", CGL_OOM: "OOM", CGL_CUDA_ERROR: "CUDA_ERROR",
    CGL_DEVICE_TIMEOUT: "DEVICE_TIMEOUT", CGL_DESTROYED: "DESTROYED", CGL_WARNING: "WARNING",
}

STAGE_GRAVITY = 1 << 0
STAGE_CENTER = 1 << 1
STAGE_MANYBODY = 1 << 2
STAGE_LINK_IN = 1 << 3
STAGE_LINK_OUT = 1 << 4
STAGE_COLLISION = 1 << 5
STAGE_CLUSTERS = 1 << 6
STAGE_ALL = 0x7F

NUM_STAGE_TIMES = 11
STAGE_TIME_NAMES = [
    "prepass", "center", "scan", "scatter", "cells", "manybody", "link_in", "link_out",
    "collision_grid", "collision_force", "clusters",
]


class Config(C.Structure):
    _fields_ = [
        ("space_size", C.c_double),
        ("simulation_decay", C.c_double),
        ("simulation_gravity", C.c_double),
        ("simulation_center", C.c_double),
        ("simulation_repulsion", C.c_double),
        ("simulation_repulsion_theta", C.c_double),
        ("simulation_link_spring", C.c_double),
        ("simulation_link_distance", C.c_double),
        ("simulation_link_dist_random_variation_range", C.c_double * 2),
        ("simulation_friction", C.c_double),
        ("simulation_collision", C.c_double),
        ("simulation_collision_radius", C.c_double),
        ("simulation_collision_padding", C.c_double),
        ("point_default_size", C.c_double),
        ("enable_simulation", C.c_int32),
        ("has_random_seed", C.c_int32),
        ("random_seed", C.c_uint64),
        ("max_texture_dimension", C.c_double),
        ("stage_mask", C.c_uint32),
        ("device", C.c_int32),
        ("hbm_budget_bytes", C.c_double),
        ("simulation_cluster", C.c_double),
        ("simulation_repulsion_from_mouse", C.c_double),
        ("enable_right_click_repulsion", C.c_int32),
        ("enable_drag", C.c_int32),
        ("device_ingest_min_links", C.c_double),
        ("random_stream", C.c_int32),
        ("rescale_positions", C.c_int32),
        ("random_seed_text", C.c_char_p),
        ("manybody_kernel", C.c_int32),
    ]


RANDOM_REFERENCE = 0
RANDOM_COUNTER = 1


class State(C.Structure):
    _fields_ = [
        ("alpha", C.c_double),
        ("progress", C.c_double),
        ("is_simulation_running", C.c_int32),
        ("destroyed", C.c_int32),
        ("tick", C.c_uint64),
        ("points_number", C.c_uint64),
        ("links_number", C.c_uint64),
        ("rng_draws", C.c_uint64),
    ]


class Layout(C.Structure):
    _fields_ = [
        ("points_number", C.c_uint64),
        ("live_points", C.c_uint64),
        ("links_number", C.c_uint64),
        ("link_entries_in", C.c_uint64),
        ("points_texture_size", C.c_uint32),
        ("finest_grid", C.c_uint32),
        ("levels", C.c_uint32),
        ("max_degree_in", C.c_uint32),
        ("max_degree_out", C.c_uint32),
        ("fixed_point_bits", C.c_int32),
        ("fixed_point_bound", C.c_float),
        ("collision_grid", C.c_uint32),
        ("collision_cell_size", C.c_float),
        ("device_bytes", C.c_uint64),
        ("kernels_per_tick", C.c_uint32),
        ("manybody_kernel", C.c_uint32),
        ("manybody_tuned", C.c_uint32),
        ("early_hubs", C.c_uint32),
        ("early_points", C.c_uint32),
        ("leading_out_hubs", C.c_uint32),
    ]


MANYBODY_AUTO = -1
MANYBODY_ONE_POINT = 0
MANYBODY_SPLIT = 1
MANYBODY_TWO_POINTS = 2
CGL_ERROR_SCAN = 1          # error bit of a one-pass cell scan whose bounded wait gave up


# Reference defaults (src/variables.ts:10,15,19,69-82,147-148) mapped to C field names.
DEFAULTS = dict(
    space_size=4096.0,
    simulation_decay=5000.0,
    simulation_gravity=0.25,
    simulation_center=0.0,
    simulation_repulsion=1.0,
    simulation_repulsion_theta=1.15,
    simulation_link_spring=1.0,
    simulation_link_distance=10.0,
    simulation_link_dist_random_variation_range=(1.0, 1.2),
    simulation_friction=0.85,
    simulation_collision=0.0,
    simulation_collision_radius=math.nan,
    simulation_collision_padding=0.0,
    point_default_size=4.0,
    enable_simulation=1,
    has_random_seed=0,
    random_seed=0,
    max_texture_dimension=0.0,
    stage_mask=STAGE_ALL,
    device=0,
    hbm_budget_bytes=0.0,
    simulation_cluster=0.1,
    simulation_repulsion_from_mouse=2.0,
    enable_right_click_repulsion=0,
    enable_drag=0,
    device_ingest_min_links=65536.0,
    random_stream=RANDOM_REFERENCE,
    rescale_positions=-1,
    random_seed_text=None,
    manybody_kernel=-1,
)

# Reference config keys (camelCase, src/config.ts) -> C field names.
CAMEL_TO_FIELD = {
    "spaceSize": "space_size",
    "simulationDecay": "simulation_decay",
    "simulationGravity": "simulation_gravity",
    "simulationCenter": "simulation_center",
    "simulationRepulsion": "simulation_repulsion",
    "simulationRepulsionTheta": "simulation_repulsion_theta",
    "simulationLinkSpring": "simulation_link_spring",
    "simulationLinkDistance": "simulation_link_distance",
    "simulationLinkDistRandomVariationRange": "simulation_link_dist_random_variation_range",
    "simulationFriction": "simulation_friction",
    "simulationCollision": "simulation_collision",
    "simulationCollisionRadius": "simulation_collision_radius",
    "simulationCollisionPadding": "simulation_collision_padding",
    "pointDefaultSize": "point_default_size",
    "enableSimulation": "enable_simulation",
    "randomSeed": "random_seed",
    "simulationCluster": "simulation_cluster",
    "simulationRepulsionFromMouse": "simulation_repulsion_from_mouse",
    "enableRightClickRepulsion": "enable_right_click_repulsion",
    "enableDrag": "enable_drag",
    "rescalePositions": "rescale_positions",
}


def js_number_to_string(x):
    """JavaScript's String(x) for a number (ECMA-262 Number::toString, radix 10)."""
    import decimal
    x = float(x)
    if x != x:
        return "NaN"
    if x == 0:
        return "0"
    if x < 0:
        return "-" + js_number_to_string(-x)
    if x == math.inf:
        return "Infinity"
    # shortest round-trip digits s (k of them) and n with x = 0.s * 10^n
    t = decimal.Decimal(repr(x)).normalize().as_tuple()
    digits = "".join(str(d) for d in t.digits)
    k = len(digits)
    n = t.exponent + k
    if k <= n <= 21:
        return digits + "0" * (n - k)
    if 0 < n <= 21:
        return digits[:n] + "." + digits[n:]
    if -6 < n <= 0:
        return "0." + "0" * (-n) + digits
    e = n - 1
    sign = "+" if e >= 0 else "-"
    mant = digits[0] + ("." + digits[1:] if k > 1 else "")
    return "%se%s%d" % (mant, sign, abs(e))


def seed_fields(seed):
    """randomSeed (a number or a string, src/config.ts:771) as config fields.

    The reference seeds its generator with String(randomSeed) (random@4.1.0's
    clone over seedrandom@3.0.5): random_seed_text carries that text whenever it
    is not simply random_seed in decimal.  random_seed also keys the engine's
    opt-in counter stream: integers modulo 2^64, other numbers by their
    IEEE-754 bits, strings by FNV-1a 64.
    """
    if isinstance(seed, bool):
        seed = int(seed)
    if isinstance(seed, int):
        if 0 <= seed < (1 << 64):
            return seed, None
        return seed % (1 << 64), str(seed)
    if isinstance(seed, float):
        text = js_number_to_string(seed)
        if seed.is_integer() and 0 <= seed < 2.0 ** 53:
            return int(seed), None
        import struct
        return struct.unpack("<Q", struct.pack("<d", seed))[0], text
    text = str(seed)
    h = 0xCBF29CE484222325
    for b in text.encode("utf-8"):
        h ^= b
        h = (h * 0x100000001B3) % (1 << 64)
    return h, text


def seed_to_u64(seed):
    """The 64-bit random_seed field for a randomSeed value (see seed_fields)."""
    return seed_fields(seed)[0]


def make_config(**fields) -> Config:
    """Build a Config from defaults plus snake_case overrides (`random_seed` sets has_random_seed)."""
    vals = dict(DEFAULTS)
    for k, v in fields.items():
        if k not in vals:
            raise KeyError("unknown config field %r" % k)
        vals[k] = v
    if "random_seed" in fields and fields["random_seed"] is not None:
        vals["has_random_seed"] = 1
        u64, text = seed_fields(fields["random_seed"])
        vals["random_seed"] = u64
        if "random_seed_text" not in fields:
            vals["random_seed_text"] = text
    elif "random_seed" in fields:
        vals["has_random_seed"] = 0
        vals["random_seed"] = 0
    if isinstance(vals.get("random_seed_text"), str):
        vals["random_seed_text"] = vals["random_seed_text"].encode("utf-8")
    cfg = Config()
    for k, v in vals.items():
        if k == "simulation_link_dist_random_variation_range":
            arr = (C.c_double * 2)(float(v[0]), float(v[1]))
            setattr(cfg, k, arr)
        else:
            setattr(cfg, k, v)
    return cfg


def config_to_dict(cfg: Config) -> dict:
    out = {}
    for name, _ in Config._fields_:
        v = getattr(cfg, name)
        if name == "simulation_link_dist_random_variation_range":
            v = (v[0], v[1])
        elif name == "random_seed_text" and v is not None:
            v = v.decode("utf-8")
        out[name] = v
    return out


def declare(lib, prefix: str, engine_t=C.c_void_p):
    """Set argtypes/restype on the engine-style API of `lib` (prefix 'cgl' or 'orc')."""
    E = engine_t
    f = C.POINTER(C.c_float)
    spec = {
        "set_point_positions": ([E, f, C.c_uint64], C.c_int),
        "set_point_positions_ex": ([E, f, C.c_uint64, C.c_int32], C.c_int),
        "set_links": ([E, f, C.c_uint64], C.c_int),
        "set_link_strength": ([E, f, C.c_uint64], C.c_int),
        "set_point_sizes": ([E, f, C.c_uint64], C.c_int),
        "set_pinned_points": ([E, C.POINTER(C.c_double), C.c_uint64], C.c_int),
        "set_point_clusters": ([E, f, C.c_uint64], C.c_int),
        "set_cluster_positions": ([E, f, C.c_uint64], C.c_int),
        "set_point_cluster_strength": ([E, f, C.c_uint64], C.c_int),
        "get_cluster_positions": ([E, C.POINTER(C.c_double), C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
        "set_pointer": ([E, C.c_double, C.c_double, C.c_int32], C.c_int),
        "set_drag": ([E, C.c_int64], C.c_int),
        "frame": ([E, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
        "render": ([E, C.c_double], C.c_int),
        "start": ([E, C.c_double], C.c_int),
        "stop": ([E], C.c_int),
        "pause": ([E], C.c_int),
        "unpause": ([E], C.c_int),
        "step": ([E, C.c_uint32], C.c_int),
        "run": ([E, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
        "get_point_positions": ([E, f, C.c_uint64], C.c_int),
        "get_state": ([E, C.POINTER(State)], C.c_int),
        "get_layout": ([E, C.POINTER(Layout)], C.c_int),
        "set_config": ([E, C.POINTER(Config)], C.c_int),
        "debug_get_cells": ([E, C.c_uint32, f, C.c_uint64], C.c_int),
        "debug_get_slots": ([E, C.POINTER(C.c_int32), C.c_uint64], C.c_int),
    }
    for name, (args, res) in spec.items():
        fn = getattr(lib, "%s_%s" % (prefix, name))
        fn.argtypes = args
        fn.restype = res


class BatchInfo(C.Structure):
    _fields_ = [
        ("jobs", C.c_uint64),
        ("running_jobs", C.c_uint64),
        ("points", C.c_uint64),
        ("link_entries", C.c_uint64),
        ("point_arena", C.c_uint64),
        ("cell_arena", C.c_uint64),
        ("device_bytes", C.c_uint64),
        ("kernels_per_tick", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class BatchJob(C.Structure):
    """cgl_batch_job (include/cgl.h): one job of cgl_batch_add_many."""
    _fields_ = [
        ("cfg", C.POINTER(Config)),
        ("xy", C.POINTER(C.c_float)),
        ("n_floats", C.c_uint64),
        ("links", C.POINTER(C.c_float)),
        ("n_link_floats", C.c_uint64),
        ("sizes", C.POINTER(C.c_float)),
        ("n_sizes", C.c_uint64),
        ("max_ticks", C.c_uint32),
        ("stop_below_alpha_min", C.c_int32),
    ]
