"""ctypes wrapper over the CPU oracle (oracle/oracle.cpp) — TEST INFRASTRUCTURE ONLY.

Imported by the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``; never by the product package.  ``build()`` compiles the oracle with g++ into
oracle/_build/liboracle.so, and the reference-derived checker into oracle/_ref/ when the
reference checkout is present (see ref_build.py).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")

_lib = None
_ref = None


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        tmp = LIB + ".tmp.%d" % os.getpid()
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
                        "-o", tmp, src], check=True)
        os.replace(tmp, LIB)
    return LIB


def build_ref():
    import ref_build  # noqa: F401  (same directory)
    return ref_build.build(quiet=True)


class ChaosCfg(ctypes.Structure):
    _fields_ = [("walkers", ctypes.c_uint64), ("temporal_samples", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("fuse_passes", ctypes.c_uint32),
                ("draw_passes", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("fp64", ctypes.c_int), ("shuffle_mode", ctypes.c_int),
                ("cta_slots", ctypes.c_uint32), ("steps_per_launch", ctypes.c_uint32),
                ("table_size", ctypes.c_uint32), ("tss_width", ctypes.c_float),
                ("threads", ctypes.c_int), ("table_seed_set", ctypes.c_int), ("table_seed", ctypes.c_uint64),
                ("badval_reset", ctypes.c_int), ("table_phases", ctypes.c_uint32)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.orc_jsf_warmup.argtypes = [ctypes.c_uint32, u32p]
        L.orc_jsf_next.argtypes = [u32p]
        L.orc_jsf_next.restype = ctypes.c_uint32
        L.orc_randf.argtypes = [u32p]
        L.orc_randf.restype = ctypes.c_float
        L.orc_sample_points.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
        L.orc_feistel.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
        L.orc_feistel.restype = ctypes.c_uint32
        L.orc_derive_key.argtypes = [ctypes.c_uint64] * 4
        L.orc_derive_key.restype = ctypes.c_uint64
        L.orc_shuffle_table.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_void_p]
        L.orc_shuffle_table.restype = None
        L.orc_genome_from_xml.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p, ctypes.c_int]
        L.orc_genome_free.argtypes = [ctypes.c_void_p]
        L.orc_genome_num_xforms.argtypes = [ctypes.c_void_p]
        L.orc_genome_has_final.argtypes = [ctypes.c_void_p]
        L.orc_genome_param_buffer.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_genome_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_genome_layout_json.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
        L.orc_animate_params.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint32,
                                         ctypes.c_void_p, ctypes.c_int]
        L.orc_de_radius.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_de_weight.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_de_weight.restype = ctypes.c_double
        L.orc_screen_affine.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
        L.orc_xform_draws.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_select_xform.argtypes = [ctypes.c_void_p, ctypes.c_float]
        L.orc_eval_xform.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_chaos.argtypes = [ctypes.c_void_p, ctypes.POINTER(ChaosCfg), ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_void_p]
        L.orc_xid_sequence.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
        L.orc_cpu_baseline.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]
        L.orc_cpu_baseline.restype = ctypes.c_uint64
        L.orc_density_estimate.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
        L.orc_tonemap.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_void_p]
        L.orc_filter_kernel.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.orc_tonemap_filter.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.orc_downsample.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_void_p]
        _lib = L
    return _lib


def ref_lib():
    """The reference-derived checker library, or None when it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        R = ctypes.CDLL(REF_LIB)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        R.ref_jsf_warmup.argtypes = [ctypes.c_uint32, u32p]
        R.ref_jsf_ranval_cpu.argtypes = [u32p]
        R.ref_jsf_ranval_cpu.restype = ctypes.c_uint32
        R.ref_sample_points.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
        R.ref_var_count.restype = ctypes.c_int
        R.ref_var_name.argtypes = [ctypes.c_int]
        R.ref_var_name.restype = ctypes.c_char_p
        ip = ctypes.POINTER(ctypes.c_int)
        R.ref_var_info.argtypes = [ctypes.c_int, ip, ip, ip, ip]
        R.ref_vary.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                               ctypes.c_void_p, u32p, ctypes.c_void_p]
        R.ref_glsl_randf.argtypes = [u32p]
        R.ref_glsl_randf.restype = ctypes.c_float
        _ref = R
    return _ref


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def jsf_warmup(seed):
    st = (ctypes.c_uint32 * 4)()
    lib().orc_jsf_warmup(seed, st)
    return np.array(list(st), dtype=np.uint32)


def randf_stream(state, n):
    st = (ctypes.c_uint32 * 4)(*[int(v) for v in state])
    out = np.array([lib().orc_randf(st) for _ in range(n)], dtype=np.float32)
    return out, np.array(list(st), dtype=np.uint32)


def sample_points(count):
    out = np.zeros((count, 4), np.float32)
    lib().orc_sample_points(count, _ptr(out))
    return out


def feistel(x, n, key):
    return lib().orc_feistel(x, n, key)


def derive_key(seed, a, b, tag):
    return lib().orc_derive_key(seed, a, b, tag)


def shuffle_table(n, count, seed, phases=0):
    """The kernel's shuffle table: `count` permutations of a CTA's n slots ([count, n] uint32)."""
    out = np.zeros((count, n), np.uint32)
    lib().orc_shuffle_table(n, count, seed, phases, _ptr(out))
    return out


class Genome:
    def __init__(self, xml):
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        if isinstance(xml, str):
            xml = xml.encode()
        if lib().orc_genome_from_xml(xml, ctypes.byref(h), err, 512) != 0:
            raise ValueError("oracle genome load failed: " + err.value.decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_genome_free(self.h)
            self.h = None

    @property
    def num_xforms(self):
        return lib().orc_genome_num_xforms(self.h)

    @property
    def has_final(self):
        return bool(lib().orc_genome_has_final(self.h))

    def param_buffer(self):
        n = lib().orc_genome_param_buffer(self.h, None, 0)
        out = np.zeros(n, np.float32)
        lib().orc_genome_param_buffer(self.h, _ptr(out), n)
        return out

    def layout(self):
        """The parameter buffer's layout as the reference's buffer_map_ (flame.cpp:33-71)."""
        import json
        n = lib().orc_genome_layout_json(self.h, None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        lib().orc_genome_layout_json(self.h, buf, n + 1)
        return json.loads(buf.value.decode())

    def animate_params(self, T, tss_width, t):
        """The flat parameter buffer of temporal sample t of T (animate.tpl.glsl)."""
        n = lib().orc_genome_param_buffer(self.h, None, 0)
        out = np.zeros(n, np.float32)
        if lib().orc_animate_params(self.h, T, tss_width, t, _ptr(out), n) != n:
            raise ValueError("animate_params failed")
        return out

    def info(self):
        o = np.zeros(12, np.float64)
        lib().orc_genome_info(self.h, _ptr(o))
        keys = ["width", "height", "center_x", "center_y", "scale", "rotate", "estimator_radius",
                "estimator_min", "estimator_curve", "gamma", "vibrancy", "brightness"]
        return dict(zip(keys, o.tolist()))

    def screen_affine(self, w, h):
        o = np.zeros(6, np.float32)
        lib().orc_screen_affine(self.h, w, h, _ptr(o))
        return o

    def xform_draws(self, xi, first_run=False):
        return lib().orc_xform_draws(self.h, xi, int(first_run))

    def select(self, r):
        return lib().orc_select_xform(self.h, r)

    def eval_xform(self, xi, xyc, rng_states, first_run=False, fp64=True):
        xyc = np.ascontiguousarray(xyc, np.float32)
        st = np.ascontiguousarray(rng_states, np.uint32).copy()
        n = xyc.shape[0]
        out = np.zeros((n, 4), np.float64)
        rc = lib().orc_eval_xform(self.h, xi, int(fp64), n, _ptr(xyc), _ptr(st), int(first_run), _ptr(out))
        if rc != 0:
            raise ValueError("eval_xform failed")
        return out, st

    def chaos(self, walkers, width, height, fuse=20, draw=16, seed=0, temporal_samples=1, fp64=True,
              shuffle_mode=0, cta_slots=1024, steps_per_launch=32, table_size=1024, tss_width=0.02,
              trace=False, want_rgba=True, table_seed=None, badval_reset=False, threads=1, table_phases=None,
              cta_threads=None):
        # the library's Sim builds its shuffle table for slots / threads phases per pass when that
        # is 4 (threads = min(slots, 1024) unless given); the batched launch's table is uniform
        if table_phases is None:
            spt = cta_slots // (cta_threads or min(cta_slots, 1024))
            table_phases = 0 if table_seed is not None or spt < 3 else spt
        cfg = ChaosCfg(walkers, temporal_samples, seed, fuse, draw, width, height, int(fp64), shuffle_mode,
                       cta_slots, steps_per_launch, table_size, tss_width, threads, int(table_seed is not None),
                       table_seed or 0, int(bool(badval_reset)), table_phases)
        rgba = np.zeros((height, width, 4), np.float64) if want_rgba else None
        hits = np.zeros((height, width), np.uint64)
        tr = np.zeros((fuse + draw, walkers // 256), np.uint8) if trace else None
        cnt = np.zeros(2, np.uint64)
        rc = lib().orc_chaos(self.h, ctypes.byref(cfg), _ptr(rgba) if rgba is not None else None, _ptr(hits),
                             _ptr(tr) if tr is not None else None, _ptr(cnt))
        if rc != 0:
            raise ValueError("oracle chaos failed (rc=%d)" % rc)
        return {"rgba": rgba, "hits": hits, "trace": tr, "drawn": int(cnt[0]), "emitted": int(cnt[1])}

    def xid_sequence(self, walkers, fuse, draw, seed=0, temporal_samples=1):
        out = np.zeros((fuse + draw, walkers // 256), np.uint8)
        rc = lib().orc_xid_sequence(self.h, walkers, temporal_samples, seed, fuse, draw, _ptr(out))
        if rc != 0:
            raise ValueError("xid_sequence failed")
        return out

    def cpu_baseline(self, walkers, passes, width, height, threads, seed=0, want=False, badval_reset=False,
                     binned=False):
        rgba = np.zeros((height, width, 4), np.float32) if want else None
        hits = np.zeros((height, width), np.uint32) if want else None
        nb = ctypes.c_uint64(0)
        n = lib().orc_cpu_baseline(self.h, walkers, passes, width, height, threads, seed, int(bool(badval_reset)),
                                   _ptr(rgba) if want else None, _ptr(hits) if want else None, ctypes.byref(nb))
        if binned:
            return n, rgba, hits, nb.value
        return n, rgba, hits


def de_radius(a, radius, min_radius, curve):
    return lib().orc_de_radius(a, radius, min_radius, curve)


def de_weight(dx, dy, r):
    """Kernel weight at offset (dx, dy) of a disc of radius r, or -1 outside it."""
    return lib().orc_de_weight(dx, dy, r)


def density_estimate(rgba, radius, min_radius, curve):
    rgba = np.ascontiguousarray(rgba, np.float64)
    h, w = rgba.shape[:2]
    out = np.zeros_like(rgba)
    if lib().orc_density_estimate(_ptr(rgba), w, h, radius, min_radius, curve, _ptr(out)) != 0:
        raise ValueError("density_estimate failed")
    return out


def tonemap(rgba, gamma, brightness, vibrancy, k2, ss=1):
    rgba = np.ascontiguousarray(rgba, np.float64)
    h, w = rgba.shape[:2]
    out = np.zeros((h // ss, w // ss, 4), np.float64)
    if lib().orc_tonemap(_ptr(rgba), w, h, ss, gamma, brightness, vibrancy, k2, _ptr(out)) != 0:
        raise ValueError("tonemap failed")
    return out


def filter_kernel(ss, radius, shape):
    taps = np.zeros(256, np.float64)
    n = lib().orc_filter_kernel(ss, radius, shape, _ptr(taps), 256)
    if n < 0:
        raise ValueError("bad filter")
    return taps[:n]


def tonemap_filter(rgba, ss, radius, shape, gamma, brightness, vibrancy, k2):
    """The tonemap with flam3's spatial filter in place of the ss x ss box."""
    rgba = np.ascontiguousarray(rgba, np.float64)
    h, w = rgba.shape[:2]
    out = np.zeros((h // ss, w // ss, 4), np.float64)
    if lib().orc_tonemap_filter(_ptr(rgba), w, h, ss, radius, shape, gamma, brightness, vibrancy, k2, _ptr(out)) != 0:
        raise ValueError("tonemap_filter failed")
    return out


def downsample(rgba, ss):
    rgba = np.ascontiguousarray(rgba, np.float64)
    h, w = rgba.shape[:2]
    out = np.zeros((h // ss, w // ss, 4), np.float64)
    if lib().orc_downsample(_ptr(rgba), w, h, ss, _ptr(out)) != 0:
        raise ValueError("downsample failed")
    return out
