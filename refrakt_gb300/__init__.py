"""refrakt_gb300 — GB300-native fractal-flame chaos game behind the reference's interface.

Python mirror of the C ABI (include/refrakt.h).  The names follow the reference's C++ classes:
``FlameCompiler`` is ``flame_compiler`` (src/variation_table.hpp:20-59); ``Flame`` holds a genome
(``flame::load_flame``, src/flame.cpp:160-226); ``Sim`` owns walkers, RNG states and the
shuffle table (``flame::set_sim_parameters``, flame.cpp:105-158) and runs ``warmup`` and
``draw_to_bins`` (flame.cpp:228-330).  Every call goes to the CUDA library; nothing here computes
on the CPU, and a missing library raises instead of falling back.

Device buffers are passed as torch CUDA tensors (or raw device addresses).
"""
import ctypes
import json
import os

__all__ = ["RefraktError", "FlameCompiler", "Flame", "Sim", "library", "build", "density_estimate",
           "tonemap", "hist_stats", "shuffle_generate", "probe_xform", "write_png", "render",
           "SYNTH_SMALL", "SYNTH_RANDOM", "SYNTH_CONTRACT", "SYNTH_SPACEFILL",
           "SPLAT_AUTO", "SPLAT_GLOBAL", "SPLAT_WARP", "BINS_AUTO", "BINS_DIRECT", "BINS_INTERLEAVED", "Batch", "Denoiser", "denoiser_features", "gemm_bf16",
           "GEMM_STORE_F32", "GEMM_STORE_BF16", "GEMM_ATOMIC_F32"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librefrakt_gb300.so")

SYNTH_SMALL, SYNTH_RANDOM, SYNTH_CONTRACT, SYNTH_SPACEFILL = 0, 1, 2, 3
SPLAT_AUTO, SPLAT_GLOBAL, SPLAT_WARP, SPLAT_TILE = 0, 1, 2, 3
EXCHANGE_BARRIER, EXCHANGE_PIPELINED, EXCHANGE_AUTO = 0, 1, 2
BINS_AUTO, BINS_DIRECT, BINS_INTERLEAVED = 0, 1, 2
FILTER_GAUSSIAN, FILTER_BOX, FILTER_TRIANGLE, FILTER_HERMITE = 0, 1, 2, 3

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "PARSE", 3: "UNKNOWN_NAME", 4: "UNSUPPORTED", 5: "CAPACITY",
          6: "CUDA", 7: "NEEDS_WARMUP", 8: "IO", 9: "NO_DEVICE"}


class RefraktError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status
        self.message = message


class SynthDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("n_xforms", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("final_xform", ctypes.c_int32), ("force_parametric", ctypes.c_int32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class FlameInfo(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32 * 2), ("center", ctypes.c_float * 2), ("scale", ctypes.c_float),
                ("rotate", ctypes.c_float), ("estimator_radius", ctypes.c_int32),
                ("estimator_min", ctypes.c_int32), ("estimator_curve", ctypes.c_float),
                ("gamma", ctypes.c_float), ("vibrancy", ctypes.c_float), ("brightness", ctypes.c_float),
                ("num_xforms", ctypes.c_uint32), ("has_final", ctypes.c_int32),
                ("total_params", ctypes.c_uint32), ("filter", ctypes.c_float), ("filter_shape", ctypes.c_int32)]


class XformDesc(ctypes.Structure):
    _fields_ = [("weight", ctypes.c_float), ("color", ctypes.c_float), ("color_speed", ctypes.c_float),
                ("opacity", ctypes.c_float), ("coefs", ctypes.c_float * 6), ("has_post", ctypes.c_int32),
                ("post", ctypes.c_float * 6), ("n_vars", ctypes.c_uint32), ("var_names", ctypes.POINTER(ctypes.c_char_p)),
                ("var_weights", ctypes.POINTER(ctypes.c_float)), ("n_params", ctypes.c_uint32),
                ("param_names", ctypes.POINTER(ctypes.c_char_p)), ("param_values", ctypes.POINTER(ctypes.c_float))]


class GenomeDesc(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32 * 2), ("center", ctypes.c_float * 2), ("scale", ctypes.c_float),
                ("rotate", ctypes.c_float), ("estimator_radius", ctypes.c_int32), ("estimator_min", ctypes.c_int32),
                ("estimator_curve", ctypes.c_float), ("gamma", ctypes.c_float), ("vibrancy", ctypes.c_float),
                ("brightness", ctypes.c_float), ("palette_rgb", ctypes.POINTER(ctypes.c_float)),
                ("n_xforms", ctypes.c_uint32), ("xforms", ctypes.POINTER(XformDesc)),
                ("final_xform", ctypes.POINTER(XformDesc))]


class SimDesc(ctypes.Structure):
    _fields_ = [("walkers", ctypes.c_uint64), ("temporal_samples", ctypes.c_uint32),
                ("shuffle_count", ctypes.c_uint32), ("seed", ctypes.c_uint64), ("cta_slots", ctypes.c_uint32),
                ("cta_threads", ctypes.c_uint32), ("steps_per_launch", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("specialize", ctypes.c_int32)]


class RenderDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("supersample", ctypes.c_uint32),
                ("fuse_passes", ctypes.c_uint32), ("points", ctypes.c_uint64), ("tss_width", ctypes.c_float),
                ("k2", ctypes.c_float), ("density_estimation", ctypes.c_int32), ("stop_on_binned", ctypes.c_int32)]


class BatchItem(ctypes.Structure):
    _fields_ = [("flame", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("supersample", ctypes.c_uint32), ("points", ctypes.c_uint64), ("seed", ctypes.c_uint64)]


class BatchDesc(ctypes.Structure):
    _fields_ = [("fuse_passes", ctypes.c_uint32), ("cta_slots", ctypes.c_uint32), ("unit_passes", ctypes.c_uint32),
                ("density_estimation", ctypes.c_int32), ("k2", ctypes.c_float), ("use_graph", ctypes.c_int32),
                ("device", ctypes.c_int32), ("splat", ctypes.c_int32), ("image_f32", ctypes.c_int32),
                ("specialize", ctypes.c_int32), ("bad_value_reset", ctypes.c_int32)]


class DenoiserDesc(ctypes.Structure):
    _fields_ = [("max_pixels", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("device", ctypes.c_int32)]


class DenoiserLayer(ctypes.Structure):
    _fields_ = [("in_a", ctypes.c_uint32), ("in_b", ctypes.c_uint32), ("out", ctypes.c_uint32),
                ("taps", ctypes.c_uint32), ("upsample", ctypes.c_int32), ("relu", ctypes.c_int32),
                ("level", ctypes.c_int32), ("src_a", ctypes.c_int32), ("src_b", ctypes.c_int32)]


_lib = None

_SIGS = {
    "rf_last_error": ([], ctypes.c_char_p),
    "rf_abi_version": ([], ctypes.c_int),
    "rf_compiler_create": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_compiler_destroy": ([ctypes.c_void_p], None),
    "rf_compiler_is_variation": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
    "rf_compiler_is_param": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
    "rf_compiler_is_common": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
    "rf_compiler_is_supported": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
    "rf_compiler_param_owner": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rf_compiler_num_variations": ([ctypes.c_void_p], ctypes.c_int),
    "rf_compiler_variation_name": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rf_compiler_variation_params": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rf_flame_load": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_flame_load_xml": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_flame_free": ([ctypes.c_void_p], None),
    "rf_flame_to_xml": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "rf_flame_synthesize": ([ctypes.POINTER(SynthDesc), ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_flame_from_struct": ([ctypes.POINTER(GenomeDesc), ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
                             ctypes.c_int),
    "rf_flame_get_info": ([ctypes.c_void_p, ctypes.POINTER(FlameInfo)], ctypes.c_int),
    "rf_flame_interpolate": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_flame_set_view": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_float], ctypes.c_int),
    "rf_flame_set_tonemap": ([ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float], ctypes.c_int),
    "rf_flame_set_estimator": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float], ctypes.c_int),
    "rf_flame_set_xform_value": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_float], ctypes.c_int),
    "rf_flame_param_buffer": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "rf_flame_param_layout": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "rf_flame_screen_affine": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "rf_flame_xform_draws": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rf_sim_create": ([ctypes.POINTER(SimDesc), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_sim_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rf_sim_set_stream": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_sim_enable_xid_trace": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int),
    "rf_sim_read_xid_trace": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "rf_needs_warmup": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_warmup": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float], ctypes.c_int),
    "rf_draw_to_bins": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                         ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "rf_set_splat": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rf_set_bad_value_reset": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rf_set_exchange": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rf_sim_exchange": ([ctypes.c_void_p], ctypes.c_int),
    "rf_sim_splat_tile": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_set_splat_tile": ([ctypes.c_void_p] + [ctypes.c_uint32] * 4, ctypes.c_int),
    "rf_set_bin_layout": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rf_sim_counters": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "rf_density_estimate": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                             ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_tonemap_filter": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                           ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_density_tonemap": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                            ctypes.c_float, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_hist_stats": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p], ctypes.c_int),
    "rf_tonemap": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                    ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_shuffle_generate": ([ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_probe_xform": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                        ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_render": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(RenderDesc), ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "rf_batch_create": ([ctypes.POINTER(BatchItem), ctypes.c_uint32, ctypes.POINTER(BatchDesc),
                         ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_batch_run": ([ctypes.c_void_p], ctypes.c_int),
    "rf_batch_sync": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "rf_batch_image": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "rf_batch_bins": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                       ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "rf_batch_read_bins": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_batch_info": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                       ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "rf_batch_image_f32": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "rf_batch_features": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_void_p],
                          ctypes.c_int),
    "rf_batch_splat": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int),
    "rf_batch_specialized": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int),
    "rf_batch_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rf_gemm_bf16": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 6 +
                     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "rf_conv3x3_bf16": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p] + [ctypes.c_uint32] * 4 +
                        [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                         ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_create": ([ctypes.POINTER(DenoiserDesc), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rf_denoiser_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_set_stream": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_sync": ([ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_num_layers": ([ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_layer": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(DenoiserLayer)], ctypes.c_int),
    "rf_denoiser_num_params": ([ctypes.c_void_p], ctypes.c_size_t),
    "rf_denoiser_get_params": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
    "rf_denoiser_set_params": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
    "rf_denoiser_gradients": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
    "rf_denoiser_features": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p,
                              ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_infer": ([ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 3 + [ctypes.c_void_p], ctypes.c_int),
    "rf_denoiser_train_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 3 +
                               [ctypes.c_float, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "rf_flame_kernel_source": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t,
                                ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "rf_flame_kernel_compile": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_size_t)],
                                ctypes.c_int),
    "rf_sim_specialized": ([ctypes.c_void_p], ctypes.c_int),
    "rf_write_png": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
}


def build(force=False):
    """Compile the CUDA library for sm_103a (refrakt_gb300/nvbuild.py)."""
    from . import nvbuild
    return nvbuild.build(force=force)


def library():
    """The loaded CUDA library.  Raises if it has not been built — there is no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("refrakt_gb300 CUDA library not built (%s); run "
                              "`python -c 'import refrakt_gb300 as r; r.build()'`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RefraktError(rc, library().rf_last_error().decode(errors="replace"))


def _ptr(x):
    """Device address of a torch tensor, an int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_cuda") and not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if hasattr(x, "is_contiguous") and not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return ctypes.c_void_p(x.data_ptr())
    raise TypeError("expected a device tensor or address, got %r" % type(x))


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return ctypes.c_void_p(s)
    return ctypes.c_void_p(s.cuda_stream)


def _string_out(fn, *args):
    need = ctypes.c_size_t(0)
    _check(fn(*args, None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(need.value)
    _check(fn(*args, buf, need.value, ctypes.byref(need)))
    return buf.value.decode()


class FlameCompiler:
    """flame_compiler (src/variation_table.hpp:20-59): the variation table.

    ``yaml_path=None`` uses the built-in copy of the reference's table; a path reads a
    variations.yaml and checks each entry against the device implementations."""

    def __init__(self, yaml_path=None):
        h = ctypes.c_void_p()
        _check(library().rf_compiler_create(yaml_path.encode() if yaml_path else None, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rf_compiler_destroy(self._h)
            self._h = None

    def is_variation(self, name):
        return bool(library().rf_compiler_is_variation(self._h, name.encode()))

    def is_param(self, name):
        return bool(library().rf_compiler_is_param(self._h, name.encode()))

    def is_common(self, name):
        return bool(library().rf_compiler_is_common(self._h, name.encode()))

    def is_supported(self, name):
        return bool(library().rf_compiler_is_supported(self._h, name.encode()))

    def param_owner(self, param):
        buf = ctypes.create_string_buffer(256)
        _check(library().rf_compiler_param_owner(self._h, param.encode(), buf, 256))
        return buf.value.decode()

    def variations(self):
        n = library().rf_compiler_num_variations(self._h)
        out = []
        buf = ctypes.create_string_buffer(256)
        for i in range(n):
            _check(library().rf_compiler_variation_name(self._h, i, buf, 256))
            out.append(buf.value.decode())
        return out

    def get_parameters_for_variation(self, name):
        buf = ctypes.create_string_buffer(1024)
        _check(library().rf_compiler_variation_params(self._h, name.encode(), buf, 1024))
        s = buf.value.decode()
        return s.split(",") if s else []


class Flame:
    """A genome (src/flame.hpp:41-61).  Construct with ``load_flame``, ``from_xml`` or ``synthesize``."""

    def __init__(self, handle, compiler):
        self._h = handle
        self._compiler = compiler

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rf_flame_free(self._h)
            self._h = None

    @classmethod
    def load_flame(cls, path, compiler):
        h = ctypes.c_void_p()
        _check(library().rf_flame_load(path.encode(), compiler._h, ctypes.byref(h)))
        return cls(h, compiler)

    @classmethod
    def from_xml(cls, xml, compiler):
        h = ctypes.c_void_p()
        _check(library().rf_flame_load_xml(xml.encode() if isinstance(xml, str) else xml, compiler._h, ctypes.byref(h)))
        return cls(h, compiler)

    @classmethod
    def from_struct(cls, compiler, genome):
        """A genome from a dict (rf_flame_from_struct): size, center, scale, rotate, estimator
        (radius, min, curve), gamma, vibrancy, brightness, palette (256 x 3), xforms and an optional
        final_xform, each {weight, color, color_speed, opacity, coefs, post?, vars: {name: weight},
        params: {name: value}}."""
        keep = []

        def xf(x):
            names = [n.encode() for n in x["vars"]]
            pn = [n.encode() for n in x.get("params", {})]
            vn = (ctypes.c_char_p * max(1, len(names)))(*names)
            vw = (ctypes.c_float * max(1, len(names)))(*x["vars"].values())
            pk = (ctypes.c_char_p * max(1, len(pn)))(*pn)
            pv = (ctypes.c_float * max(1, len(pn)))(*x.get("params", {}).values())
            keep.extend([vn, vw, pk, pv])
            post = x.get("post")
            return XformDesc(x["weight"], x.get("color", 0.0), x.get("color_speed", 0.5), x.get("opacity", 1.0),
                             (ctypes.c_float * 6)(*x["coefs"]), int(post is not None),
                             (ctypes.c_float * 6)(*(post or [1, 0, 0, 1, 0, 0])), len(names), vn, vw, len(pn), pk, pv)
        xs = (XformDesc * len(genome["xforms"]))(*[xf(x) for x in genome["xforms"]])
        fin = ctypes.pointer(xf(genome["final_xform"])) if genome.get("final_xform") else None
        pal = (ctypes.c_float * 768)(*[c for rgb in genome["palette"] for c in rgb])
        est = genome.get("estimator", (9, 0, 0.4))
        d = GenomeDesc((ctypes.c_uint32 * 2)(*genome["size"]), (ctypes.c_float * 2)(*genome.get("center", (0, 0))),
                       genome["scale"], genome.get("rotate", 0.0), est[0], est[1], est[2], genome.get("gamma", 2.2),
                       genome.get("vibrancy", 1.0), genome.get("brightness", 4.0), pal, len(genome["xforms"]), xs, fin)
        h = ctypes.c_void_p()
        _check(library().rf_flame_from_struct(ctypes.byref(d), compiler._h, ctypes.byref(h)))
        return cls(h, compiler)

    @classmethod
    def synthesize(cls, compiler, kind, seed, width, height, n_xforms=0, final_xform=False, force_parametric=False):
        d = SynthDesc(kind, n_xforms, seed, int(final_xform), int(force_parametric), width, height)
        h = ctypes.c_void_p()
        _check(library().rf_flame_synthesize(ctypes.byref(d), compiler._h, ctypes.byref(h)))
        return cls(h, compiler)

    def to_xml(self):
        return _string_out(library().rf_flame_to_xml, self._h)

    def interpolate(self, other, t):
        """Genome at t between self (t = 0) and other (t = 1)."""
        h = ctypes.c_void_p()
        _check(library().rf_flame_interpolate(self._h, other._h, t, ctypes.byref(h)))
        return Flame(h, self._compiler)

    def info(self):
        i = FlameInfo()
        _check(library().rf_flame_get_info(self._h, ctypes.byref(i)))
        return {"size": tuple(i.size), "center": tuple(i.center), "scale": i.scale, "rotate": i.rotate,
                "estimator_radius": i.estimator_radius, "estimator_min": i.estimator_min,
                "estimator_curve": i.estimator_curve, "gamma": i.gamma, "vibrancy": i.vibrancy,
                "brightness": i.brightness, "num_xforms": i.num_xforms, "has_final": bool(i.has_final),
                "total_params": i.total_params, "filter": i.filter, "filter_shape": i.filter_shape}

    def set_view(self, center, scale, rotate):
        c = (ctypes.c_float * 2)(*center)
        _check(library().rf_flame_set_view(self._h, c, scale, rotate))

    def set_tonemap(self, gamma, brightness, vibrancy):
        _check(library().rf_flame_set_tonemap(self._h, gamma, brightness, vibrancy))

    def set_estimator(self, radius, min_radius, curve):
        _check(library().rf_flame_set_estimator(self._h, radius, min_radius, curve))

    def set_xform_value(self, xform, name, value):
        _check(library().rf_flame_set_xform_value(self._h, xform, name.encode(), value))

    def param_buffer(self):
        import numpy as np
        n = ctypes.c_size_t(0)
        _check(library().rf_flame_param_buffer(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.float32)
        _check(library().rf_flame_param_buffer(self._h, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n)))
        return out

    def param_layout(self):
        return json.loads(_string_out(library().rf_flame_param_layout, self._h))

    def screen_affine(self, width, height):
        out = (ctypes.c_float * 6)()
        _check(library().rf_flame_screen_affine(self._h, width, height, out))
        return list(out)

    def kernel_source(self, cta_threads=1024, cta_slots=4096):
        """CUDA source of this genome's specialised chaos kernel."""
        n = ctypes.c_size_t()
        _check(library().rf_flame_kernel_source(self._h, cta_threads, cta_slots, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(library().rf_flame_kernel_source(self._h, cta_threads, cta_slots, buf, n.value, None))
        return buf.value.decode()

    def kernel_compile(self, cta_threads=1024, cta_slots=4096):
        """Compiles the specialised kernel for sm_103a (no device needed); returns the cubin size."""
        n = ctypes.c_size_t()
        _check(library().rf_flame_kernel_compile(self._h, cta_threads, cta_slots, ctypes.byref(n)))
        return n.value

    def xform_draws(self, xform):
        return library().rf_flame_xform_draws(self._h, xform)


class Sim:
    """Walker slots, RNG states and the shuffle table — ``flame::set_sim_parameters`` plus the
    per-flame ``warmup`` / ``draw_to_bins`` (src/flame.cpp:105-330)."""

    def __init__(self, walkers, temporal_samples=1, shuffle_count=1024, seed=0, cta_slots=4096, cta_threads=0,
                 steps_per_launch=0, device=0, specialize=0):
        d = SimDesc(walkers, temporal_samples, shuffle_count, seed, cta_slots, cta_threads, steps_per_launch, device,
                    specialize)
        h = ctypes.c_void_p()
        _check(library().rf_sim_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.walkers = walkers

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rf_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream):
        _check(library().rf_sim_set_stream(self._h, _stream(stream)))

    def specialized(self):
        """True when the launches after the last warmup use a genome-specialised kernel."""
        return bool(library().rf_sim_specialized(self._h))

    def enable_xid_trace(self, passes):
        _check(library().rf_sim_enable_xid_trace(self._h, passes))

    def read_xid_trace(self, passes):
        import numpy as np
        groups = self.walkers // 256
        out = np.zeros((passes, groups), np.uint8)
        got = ctypes.c_uint32(0)
        _check(library().rf_sim_read_xid_trace(self._h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes, ctypes.byref(got)))
        return out

    def needs_warmup(self, flame):
        return bool(library().rf_needs_warmup(self._h, flame._h))

    def warmup(self, flame, num_passes, tss_width=0.02):
        _check(library().rf_warmup(self._h, flame._h, num_passes, tss_width))

    def set_splat(self, splat):
        _check(library().rf_set_splat(self._h, splat))

    def set_splat_tile(self, x0, y0, w, h):
        """The bins of the shared-memory histogram tile (rf_set_splat_tile; used with SPLAT_TILE)."""
        _check(library().rf_set_splat_tile(self._h, x0, y0, w, h))

    def set_bad_value_reset(self, on):
        """Restart walkers that leave the plane (rf_set_bad_value_reset; the reference keeps this
        step commented out at shaders/flame.glsl:68, so the default is off)."""
        _check(library().rf_set_bad_value_reset(self._h, int(bool(on))))

    def set_exchange(self, mode):
        """Walker exchange of the specialised chaos kernel (rf_set_exchange): EXCHANGE_BARRIER,
        EXCHANGE_PIPELINED or EXCHANGE_AUTO (default: the faster of the two, timed on the first
        two drawing launches of >= 32 passes); every form gives the same results."""
        _check(library().rf_set_exchange(self._h, int(mode)))

    def exchange(self):
        """The form the next drawing launch runs: EXCHANGE_BARRIER or EXCHANGE_PIPELINED."""
        return library().rf_sim_exchange(self._h)

    def splat_tile(self):
        """(x0, y0, w, h) of the shared-memory tile the drawing passes use, or None."""
        t = (ctypes.c_uint32 * 4)()
        return tuple(t) if library().rf_sim_splat_tile(self._h, t) == 1 else None

    def set_bin_layout(self, layout):
        """BINS_AUTO, BINS_DIRECT or BINS_INTERLEAVED (rf_set_bin_layout)."""
        _check(library().rf_set_bin_layout(self._h, layout))

    def draw_to_bins(self, flame, bins_rgba, bins_hits, width, height, num_iter, sync=True):
        drawn = ctypes.c_uint64(0)
        _check(library().rf_draw_to_bins(self._h, flame._h, _ptr(bins_rgba), _ptr(bins_hits), width, height,
                                          num_iter, ctypes.byref(drawn) if sync else None))
        return drawn.value if sync else None

    def counters(self):
        out = (ctypes.c_uint64 * 3)()
        _check(library().rf_sim_counters(self._h, out))
        return {"drawn": out[0], "emitted": out[1], "steps": out[2]}

    def render(self, flame, width, height, points, supersample=1, fuse_passes=20, tss_width=0.0, k2=0.0,
               density_estimation=True, out=None, stop_on_binned=False):
        """One frame from genome to host RGBA8 (rf_render).  Returns (image, stats).  With
        stop_on_binned, `points` counts binned points (the reference's quality stop) instead of
        walker-steps."""
        import numpy as np
        img = out if out is not None else np.zeros((height, width, 4), np.uint8)
        d = RenderDesc(width, height, supersample, fuse_passes, points, tss_width, k2, int(density_estimation),
                       int(stop_on_binned))
        st = (ctypes.c_double * 3)()
        _check(library().rf_render(self._h, flame._h, ctypes.byref(d), img.ctypes.data_as(ctypes.c_void_p), st))
        return img, {"points": st[0], "binned": st[1], "ms": st[2]}


class Batch:
    """Many genomes drawn by one persistent launch, then density-estimated and tonemapped each
    (rf_batch_*).  `items` holds (flame, width, height, points, seed) or
    (flame, width, height, points, seed, supersample) tuples."""

    def __init__(self, items, fuse_passes=20, cta_slots=0, unit_passes=0, density_estimation=True, k2=0.0,
                 use_graph=True, device=0, splat=0, image_f32=False, specialize=0, bad_value_reset=False):
        arr = (BatchItem * len(items))()
        self.sizes = []
        self._flames = [it[0] for it in items]  # keep the genomes alive as long as the batch
        for i, it in enumerate(items):
            flame, w, h, points, seed = it[:5]
            ss = it[5] if len(it) > 5 else 1
            arr[i] = BatchItem(flame._h, w, h, ss, points, seed)
            self.sizes.append((w, h, ss))
        d = BatchDesc(fuse_passes, cta_slots, unit_passes, int(density_estimation), k2, int(use_graph), device, splat,
                      int(image_f32), specialize, int(bool(bad_value_reset)))
        h = ctypes.c_void_p()
        _check(library().rf_batch_create(arr, len(items), ctypes.byref(d), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            library().rf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self):
        _check(library().rf_batch_run(self._h))

    def sync(self):
        st = (ctypes.c_double * 4)()
        _check(library().rf_batch_sync(self._h, st))
        return {"points": st[0], "binned": st[1], "ms": st[2], "steps": st[3]}

    def image(self, i, out=None):
        import numpy as np
        w, h, _ = self.sizes[i]
        img = out if out is not None else np.zeros((h, w, 4), np.uint8)
        _check(library().rf_batch_image(self._h, i, img.ctypes.data_as(ctypes.c_void_p)))
        return img

    def image_f32(self, i, out):
        """Item i's FP32 tonemapped RGBA image into `out` (a [h, w, 4] float32 CUDA tensor or array)."""
        _check(library().rf_batch_image_f32(self._h, i, _ptr(out)))

    def features(self, i, out, k2=0.0, level=0.0):
        """Item i's learned-DE input features into `out` (a [h*ss, w*ss, 8] bf16 CUDA tensor)."""
        _check(library().rf_batch_features(self._h, i, k2, level, _ptr(out)))

    def bins(self, i):
        """Host copies of item i's RGBA sums (H, W, 4 float32) and hit counts (H, W uint32)."""
        import numpy as np
        w, h, ss = self.sizes[i]
        rgba = np.zeros((h * ss, w * ss, 4), np.float32)
        hits = np.zeros((h * ss, w * ss), np.uint32)
        _check(library().rf_batch_read_bins(self._h, i, rgba.ctypes.data_as(ctypes.c_void_p),
                                            hits.ctypes.data_as(ctypes.c_void_p)))
        return rgba, hits

    def info(self):
        a, b, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(library().rf_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"cta_slots": a.value, "units": b.value, "unit_passes": c.value,
                "splat": [library().rf_batch_splat(self._h, i) for i in range(len(self.sizes))],
                "specialized": [library().rf_batch_specialized(self._h, i) for i in range(len(self.sizes))]}


def render(sim, flame, *a, **k):
    return sim.render(flame, *a, **k)


def density_estimate(bins_rgba, width, height, radius, min_radius, curve, out, stream=None):
    _check(library().rf_density_estimate(_ptr(bins_rgba), width, height, radius, min_radius, curve, _ptr(out),
                                         _stream(stream)))


def tonemap_filter(rgba, width, height, ss, radius, shape, gamma, brightness, vibrancy, k2, out_f32=None,
                   out_rgba8=None, stream=None):
    """The tonemap with flam3's spatial filter (FILTER_GAUSSIAN ...) in place of the box (rf_tonemap_filter)."""
    _check(library().rf_tonemap_filter(_ptr(rgba), width, height, ss, radius, shape, gamma, brightness, vibrancy, k2,
                                       _ptr(out_f32), _ptr(out_rgba8), _stream(stream)))


def density_tonemap(bins_rgba, width, height, radius, min_radius, curve, ss, gamma, brightness, vibrancy, k2,
                    out_f32=None, out_rgba8=None, stream=None):
    """Density estimation then the tonemap in one call (rf_density_tonemap)."""
    _check(library().rf_density_tonemap(_ptr(bins_rgba), width, height, radius, min_radius, curve, ss, gamma,
                                        brightness, vibrancy, k2, _ptr(out_f32), _ptr(out_rgba8), _stream(stream)))


def hist_stats(rgba, width, height, stream=None):
    out = (ctypes.c_double * 3)()
    _check(library().rf_hist_stats(_ptr(rgba), width, height, out, _stream(stream)))
    return {"sum": out[0], "max": out[1], "nonzero": int(out[2])}


def tonemap(rgba, width, height, ss, gamma, brightness, vibrancy, k2, out_f32=None, out_rgba8=None, stream=None):
    _check(library().rf_tonemap(_ptr(rgba), width, height, ss, gamma, brightness, vibrancy, k2, _ptr(out_f32),
                                _ptr(out_rgba8), _stream(stream)))


def shuffle_generate(n, count, seed, out, stream=None):
    _check(library().rf_shuffle_generate(n, count, seed, _ptr(out), _stream(stream)))


def probe_xform(flame, xform, xyc, rng, out, first_run=False, stream=None):
    n = xyc.shape[0]
    _check(library().rf_probe_xform(flame._h, xform, n, _ptr(xyc), _ptr(rng), int(first_run), _ptr(out),
                                    _stream(stream)))


GEMM_STORE_F32, GEMM_STORE_BF16, GEMM_ATOMIC_F32 = 0, 1, 2


def _rows_ptr(x):
    """Device address of a 2-D CUDA tensor whose rows are contiguous (any row stride)."""
    if x.dim() != 2 or not x.is_cuda or x.stride(1) != 1:
        raise ValueError("expected a 2-D CUDA tensor with contiguous rows")
    return ctypes.c_void_p(x.data_ptr())


def gemm_bf16(a, b, c, mode=GEMM_STORE_F32, bias=None, relu=False, splits=1, stream=None):
    """c (+)= a @ b.T on the tensor cores; a (M x K) and b (N x K) bf16 CUDA tensors with
    contiguous rows (row strides multiples of 8 elements)."""
    M, K = a.shape
    N = b.shape[0]
    _check(library().rf_gemm_bf16(_rows_ptr(a), _rows_ptr(b), _rows_ptr(c), M, N, K, a.stride(0), b.stride(0),
                                  c.stride(0), mode, _ptr(bias), int(relu), splits, _stream(stream)))


def conv3x3_bf16(xa, w, c, xb=None, up=False, mode=GEMM_STORE_F32, bias=None, relu=False, stream=None):
    """c (+)= conv3x3(concat(upsample(xa) if up else xa, xb)) · w as an implicit GEMM on the tensor
    cores.  xa [n, h, w, ca] (or [n, h/2, w/2, ca] with up) and xb [n, h, w, cb] contiguous NHWC
    bf16; w [N, 9 (ca + cb)] bf16, column k = tap (ca + cb) + channel, tap = (dy + 1) 3 + (dx + 1);
    c [n h w, N] with contiguous rows."""
    n, ha, wa, ca = xa.shape
    h, wd = (2 * ha, 2 * wa) if up else (ha, wa)
    cb = 0 if xb is None else xb.shape[3]
    if w.shape[1] != 9 * (ca + cb):
        raise ValueError("conv3x3_bf16: weights must have 9 (ca + cb) = %d columns" % (9 * (ca + cb)))
    _check(library().rf_conv3x3_bf16(_ptr(xa), ca, int(up), _ptr(xb), cb, n, h, wd, _rows_ptr(w), w.shape[0],
                                     w.stride(0), _rows_ptr(c), c.stride(0), mode, _ptr(bias), int(relu),
                                     _stream(stream)))


class Denoiser:
    """The learned density estimator (rf_denoiser_*): features [n, h, w, 8] bf16 and images /
    targets [n, h, w, 3] float32 are CUDA tensors (h, w multiples of 8)."""

    def __init__(self, max_pixels, seed=0, device=0):
        h = ctypes.c_void_p()
        _check(library().rf_denoiser_create(ctypes.byref(DenoiserDesc(max_pixels, seed, device)), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            library().rf_denoiser_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream):
        _check(library().rf_denoiser_set_stream(self._h, _stream(stream)))

    def layers(self):
        out = []
        for i in range(library().rf_denoiser_num_layers(self._h)):
            li = DenoiserLayer()
            _check(library().rf_denoiser_layer(self._h, i, ctypes.byref(li)))
            out.append({k: getattr(li, k) for k, _ in DenoiserLayer._fields_})
        return out

    def num_params(self):
        return library().rf_denoiser_num_params(self._h)

    def params(self):
        import numpy as np
        a = np.zeros(self.num_params(), np.float32)
        _check(library().rf_denoiser_get_params(self._h, a.ctypes.data_as(ctypes.c_void_p), a.size))
        return a

    def set_params(self, a):
        import numpy as np
        a = np.ascontiguousarray(a, np.float32)
        _check(library().rf_denoiser_set_params(self._h, a.ctypes.data_as(ctypes.c_void_p), a.size))

    def gradients(self):
        import numpy as np
        a = np.zeros(self.num_params(), np.float32)
        _check(library().rf_denoiser_gradients(self._h, a.ctypes.data_as(ctypes.c_void_p), a.size))
        return a

    def infer(self, feats, out, sync=True):
        """out = clamp(base + net(feats)); runs on the denoiser's stream and, with sync, waits
        for it (the caller's stream may read `out` only after that)."""
        n, h, w = feats.shape[:3]
        _check(library().rf_denoiser_infer(self._h, _ptr(feats), n, h, w, _ptr(out)))
        if sync:
            _check(library().rf_denoiser_sync(self._h))

    def train_step(self, feats, target, lr):
        n, h, w = feats.shape[:3]
        loss = ctypes.c_double()
        _check(library().rf_denoiser_train_step(self._h, _ptr(feats), _ptr(target), n, h, w, lr, ctypes.byref(loss)))
        return loss.value


def denoiser_features(bins_rgba, width, height, out, k2=0.0, base=None, level=0.0, stream=None):
    _check(library().rf_denoiser_features(_ptr(bins_rgba), width, height, k2, _ptr(base), level, _ptr(out),
                                          _stream(stream)))


def write_png(path, rgba8):
    import numpy as np
    a = np.ascontiguousarray(rgba8, np.uint8)
    h, w = a.shape[:2]
    _check(library().rf_write_png(path.encode(), a.ctypes.data_as(ctypes.c_void_p), w, h))
