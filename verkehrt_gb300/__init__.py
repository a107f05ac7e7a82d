"""verkehrt_gb300: the GB300 `cuda` kernel backend of the verkehrt array language.

The compute path is libvkcuda.so (hand-written sm_103a kernels behind the C ABI declared in
include/vkcuda.h). This module is a thin ctypes host over that ABI, shaped like the reference's
kernel table (src/kernels.rs Registry / KernelDef) and Dispatch (src/kernels/dispatch.rs):

    ctx = Context()                                  # Registry::resolve for the cuda ISA
    x = ctx.call("rand_f64", 1_000_000, 1)           # Dispatch::call by kernel name
    ctx.call("dot_f64", x, ctx.call("rand_f64", 1_000_000, 2))
    r = ctx.reducer("reduce_add_f64"); r.update(x); r.finish()   # Dispatch::reducer

Kernel errors raise KernelError with the reference's message text. There is no CPU fallback:
when the library is missing or no device is present, the calls raise.
"""

import ctypes
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvkcuda.so")

# vkc_type, include/vkcuda.h; element types of src/value.rs ScalarType::ARRAY_TYPES.
TYPES = {"f64": 0, "f32": 1, "i64": 2, "u64": 3, "i32": 4, "u8": 5, "bool": 6}
TYPE_NAMES = {v: k for k, v in TYPES.items()}
NP_DTYPES = {"f64": np.float64, "f32": np.float32, "i64": np.int64, "u64": np.uint64,
             "i32": np.int32, "u8": np.uint8, "bool": np.uint8}
CLASSES = {0: "elementwise", 1: "reduction", 2: "selection", 3: "scan", 4: "whole"}
STATUS = {0: "OK", 1: "RUNTIME", 2: "ALLOC", 3: "TIMEOUT", 4: "DEVICE", 5: "USAGE"}


class KernelError(Exception):
    """A failed call: `status` is the vkc_status name, `message` the error text."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status
        self.message = message


class _Scalar(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("bits", ctypes.c_uint64)]


class _Value(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("array", ctypes.c_void_p), ("scalar", _Scalar),
                ("str", ctypes.c_char_p)]


# Every entry point of include/vkcuda.h with its ctypes signature.
_P = ctypes.c_void_p
_SIGNATURES = {
    "vkc_open": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "vkc_close": (None, [_P]),
    "vkc_last_error": (ctypes.c_char_p, [_P]),
    "vkc_synchronize": (ctypes.c_int, [_P]),
    "vkc_set_cache_limit": (ctypes.c_int, [_P, ctypes.c_size_t]),
    "vkc_tune_set": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "vkc_load_column_words": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "vkc_load_column_bytes": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_P)]),
    "vkc_tune_get": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "vkc_set_stream": (ctypes.c_int, [_P, _P]),
    "vkc_get_stream": (_P, [_P]),
    "vkc_launch_count": (ctypes.c_uint64, [_P]),
    "vkc_timer_start": (ctypes.c_int, [_P]),
    "vkc_timer_stop": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    "vkc_array_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, ctypes.POINTER(_P)]),
    "vkc_array_upload": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_int64, ctypes.POINTER(_P)]),
    "vkc_array_download": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64]),
    "vkc_array_download_start": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.POINTER(_P)]),
    "vkc_copy_wait": (ctypes.c_int, [_P, _P]),
    "vkc_array_slice": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(_P)]),
    "vkc_array_len": (ctypes.c_int64, [_P]),
    "vkc_array_type": (ctypes.c_int, [_P]),
    "vkc_array_device_ptr": (_P, [_P]),
    "vkc_array_retain": (None, [_P]),
    "vkc_array_release": (None, [_P]),
    "vkc_kernel_count": (ctypes.c_int, []),
    "vkc_kernel_name": (ctypes.c_char_p, [ctypes.c_int]),
    "vkc_kernel_lookup": (ctypes.c_int, [ctypes.c_char_p]),
    "vkc_kernel_class": (ctypes.c_int, [ctypes.c_int]),
    "vkc_kernel_arity": (ctypes.c_int, [ctypes.c_int]),
    "vkc_kernel_cost": (ctypes.c_uint64, [ctypes.c_int]),
    "vkc_call": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int,
                                ctypes.POINTER(_Value)]),
    "vkc_call_into": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int, _P,
                                     ctypes.c_int64]),
    "vkc_reducer_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    "vkc_reducer_update": (ctypes.c_int, [_P, ctypes.POINTER(_Value), ctypes.c_int]),
    "vkc_reducer_finish": (ctypes.c_int, [_P, ctypes.POINTER(_Scalar)]),
    "vkc_reducer_free": (None, [_P]),
    "vkc_scanner_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    "vkc_scanner_update": (ctypes.c_int, [_P, ctypes.POINTER(_Value), ctypes.c_int, _P]),
    "vkc_scanner_free": (None, [_P]),
    "vkc_builder_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    "vkc_builder_finish": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "vkc_builder_free": (None, [_P]),
    "vkc_select_tile": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int,
                                       ctypes.c_int64, _P]),
    "vkc_elementwise_tile": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int,
                                            _P]),
    "vkc_scan_add_i64_noalloc": (ctypes.c_int, [ctypes.c_int, _P, _P, ctypes.c_int64, _P,
                                                ctypes.c_char_p, ctypes.c_size_t]),
    "vkc_region_eval": (ctypes.c_int, [_P, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int,
                                       ctypes.POINTER(_Value)]),
    "vkc_region_reduce": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Value), ctypes.c_int,
                                         ctypes.POINTER(_Value)]),
    "vkc_batch_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "vkc_batch_free": (None, [_P]),
    "vkc_batch_len": (ctypes.c_int, [_P]),
    "vkc_batch_filter_sum_f64": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_double, _P]),
    "vkc_batch_argsort_i64": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint]),
    "vkc_batch_count_f64": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_double, _P]),
    "vkc_batch_dot_f64": (ctypes.c_int, [_P, _P, _P, _P]),
    "vkc_batch_concat": (ctypes.c_int, [_P, _P, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "vkc_batch_rand": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_P)]),
    "vkc_graph_begin": (ctypes.c_int, [_P]),
    "vkc_graph_end": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "vkc_graph_launch": (ctypes.c_int, [_P, _P]),
    "vkc_graph_free": (None, [_P]),
}



class _RegionKernel(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int32), ("nargs", ctypes.c_int32), ("args", ctypes.c_int32 * 3)]


def region_kernel(k):
    """The source naming region kernel k's output."""
    return -1 - k


_lib = None


def library_path():
    return LIB_PATH


def load():
    """Loads libvkcuda.so. Raises when it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libvkcuda.so is not built; run verkehrt_gb300.build.build() "
            "(the CUDA library is the only compute path)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGNATURES)


def kernels():
    """The kernel table: list of (name, class, arity, cost)."""
    lib = load()
    out = []
    for i in range(lib.vkc_kernel_count()):
        out.append((lib.vkc_kernel_name(i).decode(), CLASSES[lib.vkc_kernel_class(i)],
                    lib.vkc_kernel_arity(i), lib.vkc_kernel_cost(i)))
    return out


class Scalar:
    """A typed scalar argument (Arg::Splat). Python floats map to f64, ints to i64, bools to bool."""

    def __init__(self, type_name, value):
        self.type = type_name
        self.value = value

    def to_c(self):
        t = self.type
        if t == "f64":
            bits = struct.unpack("<Q", struct.pack("<d", float(self.value)))[0]
        elif t == "f32":
            bits = struct.unpack("<I", struct.pack("<f", float(self.value)))[0]
        elif t == "bool":
            bits = 1 if self.value else 0
        else:
            bits = int(self.value) & 0xFFFFFFFFFFFFFFFF
        return _Scalar(TYPES[t], bits)


def _scalar_from_c(s):
    t = TYPE_NAMES[s.type]
    b = s.bits
    if t == "f64":
        return struct.unpack("<d", struct.pack("<Q", b))[0]
    if t == "f32":
        return struct.unpack("<f", struct.pack("<I", b & 0xFFFFFFFF))[0]
    if t == "bool":
        return bool(b & 1)
    if t == "i64":
        return b - (1 << 64) if b >> 63 else b
    if t == "i32":
        b &= 0xFFFFFFFF
        return b - (1 << 32) if b >> 31 else b
    return b


def _scalar_bits_value(s):
    """(type, value, raw bits) of a returned scalar."""
    return TYPE_NAMES[s.type], _scalar_from_c(s), s.bits


class Array:
    """A device-resident array handle (src/value.rs Array). Released when collected."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h and _lib is not None:
            _lib.vkc_array_release(h)

    def __len__(self):
        return int(_lib.vkc_array_len(self.handle))

    @property
    def type(self):
        return TYPE_NAMES[_lib.vkc_array_type(self.handle)]

    @property
    def device_ptr(self):
        return _lib.vkc_array_device_ptr(self.handle)

    def numpy(self):
        n = len(self)
        out = np.empty(n, dtype=NP_DTYPES[self.type])
        if n:
            self.ctx._check(_lib.vkc_array_download(self.ctx.handle, self.handle,
                                                    out.ctypes.data_as(_P), n))
        if self.type == "bool":
            return out.astype(bool)
        return out

    def slice(self, start, end):
        h = _P()
        self.ctx._check(_lib.vkc_array_slice(self.ctx.handle, self.handle, start, end - start,
                                             ctypes.byref(h)))
        return Array(self.ctx, h.value)


class Copy:
    """An asynchronous download in flight (Context.download_start)."""

    def __init__(self, ctx, handle):
        self.ctx, self.handle = ctx, handle

    def wait(self):
        if self.handle:
            h, self.handle = self.handle, None
            self.ctx._check(_lib.vkc_copy_wait(self.ctx.handle, h))

    def __del__(self):
        try:
            self.wait()
        except Exception:
            pass


class Context:
    """A device context (one stream, one scratch arena): the cuda ISA of one interpreter."""

    def __init__(self, device=0):
        lib = load()
        h = _P()
        st = lib.vkc_open(device, ctypes.byref(h))
        if st != 0:
            raise KernelError(STATUS[st], "cannot open CUDA device %d" % device)
        self.handle = h.value
        self.device = device
        self._ids = {}

    def close(self):
        if self.handle:
            _lib.vkc_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            msg = _lib.vkc_last_error(self.handle).decode()
            raise KernelError(STATUS.get(st, str(st)), msg)

    def kernel_id(self, name):
        if name not in self._ids:
            i = _lib.vkc_kernel_lookup(name.encode())
            if i < 0:
                raise KernelError("USAGE", "no cuda entry for kernel %s" % name)
            self._ids[name] = i
        return self._ids[name]

    # ---------------------------------------------------------------- arrays

    def upload(self, values, type_name=None):
        a = np.asarray(values)
        if type_name is None:
            type_name = {np.dtype(np.float64): "f64", np.dtype(np.int64): "i64",
                         np.dtype(np.bool_): "bool", np.dtype(np.uint8): "u8",
                         np.dtype(np.uint64): "u64", np.dtype(np.int32): "i32",
                         np.dtype(np.float32): "f32"}[a.dtype]
        a = np.ascontiguousarray(a.astype(NP_DTYPES[type_name], copy=False))
        h = _P()
        self._check(_lib.vkc_array_upload(self.handle, TYPES[type_name], a.ctypes.data_as(_P),
                                          len(a), ctypes.byref(h)))
        return Array(self, h.value)

    def upload_ptr(self, ptr, n, type_name):
        """Uploads n rows from host address `ptr` (pinned memory for full-speed copies)."""
        h = _P()
        self._check(_lib.vkc_array_upload(self.handle, TYPES[type_name], ptr, n, ctypes.byref(h)))
        return Array(self, h.value)

    def download_ptr(self, arr, ptr, capacity):
        """Copies up to `capacity` rows of `arr` to host address `ptr`; waits for the copy."""
        self._check(_lib.vkc_array_download(self.handle, arr.handle, ptr, capacity))

    def download_start(self, arr, ptr, capacity):
        """Starts the same copy on the download stream (after the work queued so far) and
        returns a Copy whose wait() waits for it; uploads, kernels and other downloads overlap."""
        h = _P()
        self._check(_lib.vkc_array_download_start(self.handle, arr.handle, ptr, capacity, ctypes.byref(h)))
        return Copy(self, h.value)

    def new_array(self, type_name, n):
        h = _P()
        self._check(_lib.vkc_array_new(self.handle, TYPES[type_name], n, ctypes.byref(h)))
        return Array(self, h.value)

    # ---------------------------------------------------------------- entries

    def _values(self, args):
        vals = (_Value * max(1, len(args)))()
        for i, a in enumerate(args):
            if isinstance(a, (str, os.PathLike)):
                vals[i].kind = 2  # Value::Str: a path argument (load_T)
                vals[i].str = os.fsencode(a)
            elif isinstance(a, Array):
                vals[i].kind = 0
                vals[i].array = a.handle
            else:
                if isinstance(a, Scalar):
                    s = a
                elif isinstance(a, bool):
                    s = Scalar("bool", a)
                elif isinstance(a, (int, np.integer)):
                    s = Scalar("i64", int(a))
                else:
                    s = Scalar("f64", float(a))
                vals[i].kind = 1
                vals[i].scalar = s.to_c()
        return vals

    def call(self, name, *args, raw=False):
        """Dispatch::call: an Array for array results, a Python scalar otherwise (or the
        (type, value, bits) triple with raw=True)."""
        vals = self._values(args)
        out = _Value()
        self._check(_lib.vkc_call(self.handle, self.kernel_id(name), vals, len(args),
                                  ctypes.byref(out)))
        if out.kind == 0:
            return Array(self, out.array)
        return _scalar_bits_value(out.scalar) if raw else _scalar_from_c(out.scalar)

    def call_into(self, name, *args, out, row=0):
        """A reduction whose result goes to row `row` of the device array `out`, enqueued only
        (vkc_call_into), so it can be captured in a graph."""
        vals = self._values(args)
        self._check(_lib.vkc_call_into(self.handle, self.kernel_id(name), vals, len(args), out.handle,
                                       int(row)))

    def _region_kernels(self, kernels):
        ks = (_RegionKernel * max(1, len(kernels)))()
        for i, (name, srcs) in enumerate(kernels):
            ks[i].kernel = self.kernel_id(name)
            ks[i].nargs = len(srcs)
            for j, a in enumerate(srcs):
                ks[i].args[j] = a
        return ks

    def region(self, kernels, inputs, raw=False):
        """A region (vkc_region_eval): `kernels` in post-order as (name, sources), a source being an
        input position i >= 0 or region_kernel(k) for kernel k's output; the last kernel's value."""
        vals = self._values(inputs)
        out = _Value()
        self._check(_lib.vkc_region_eval(self.handle, ctypes.cast(self._region_kernels(kernels), ctypes.c_void_p),
                                         len(kernels), vals, len(inputs), ctypes.byref(out)))
        if out.kind == 0:
            return Array(self, out.array)
        return _scalar_bits_value(out.scalar) if raw else _scalar_from_c(out.scalar)

    def region_reduce(self, root, root_args, kernels, inputs, raw=False):
        """A fused region (vkc_region_reduce): reduction `root` over `root_args` (sources)."""
        vals = self._values(inputs)
        ra = (ctypes.c_int32 * max(1, len(root_args)))(*root_args)
        out = _Value()
        self._check(_lib.vkc_region_reduce(self.handle, self.kernel_id(root), ra, len(root_args),
                                           ctypes.cast(self._region_kernels(kernels), ctypes.c_void_p), len(kernels),
                                           vals, len(inputs), ctypes.byref(out)))
        if out.kind == 0:
            return Array(self, out.array)
        return _scalar_bits_value(out.scalar) if raw else _scalar_from_c(out.scalar)

    def reducer(self, name):
        return Reducer(self, name)

    def scanner(self, name):
        return Scanner(self, name)

    def builder(self, type_name):
        return Builder(self, type_name)

    def select_tile(self, name, args, base, builder):
        vals = self._values(args)
        self._check(_lib.vkc_select_tile(self.handle, self.kernel_id(name), vals, len(args),
                                         base, builder.handle))

    def elementwise_tile(self, name, args, out):
        vals = self._values(args)
        self._check(_lib.vkc_elementwise_tile(self.handle, self.kernel_id(name), vals, len(args),
                                              out.handle))

    # ---------------------------------------------------------------- timing and stats

    def synchronize(self):
        self._check(_lib.vkc_synchronize(self.handle))

    def set_cache_limit(self, nbytes):
        self._check(_lib.vkc_set_cache_limit(self.handle, int(nbytes)))

    def load_column_words(self, path, type_name, flip_sign=False):
        """src/columns.rs load_words: a .u64/.ends file as i64 or u64 rows on the device."""
        h = _P()
        self._check(_lib.vkc_load_column_words(self.handle, os.fsencode(path), TYPES[type_name], int(flip_sign),
                                               ctypes.byref(h)))
        return Array(self, h.value)

    def load_column_bytes(self, ends_path, bytes_path, column):
        """src/columns.rs load_single_bytes: a one-byte-per-row string column as u8 rows."""
        h = _P()
        self._check(_lib.vkc_load_column_bytes(self.handle, os.fsencode(ends_path), os.fsencode(bytes_path),
                                               column.encode(), ctypes.byref(h)))
        return Array(self, h.value)

    def tune_set(self, knob, size_class, value):
        """Overrides one entry of the autotuner table for this context (vkc_tune_set)."""
        self._check(_lib.vkc_tune_set(self.handle, knob.encode(), int(size_class), int(value)))

    def tune_get(self, knob, size_class):
        v = ctypes.c_int()
        self._check(_lib.vkc_tune_get(self.handle, knob.encode(), int(size_class), ctypes.byref(v)))
        return v.value

    def launch_count(self):
        return int(_lib.vkc_launch_count(self.handle))

    def timer_start(self):
        self._check(_lib.vkc_timer_start(self.handle))

    def timer_stop(self):
        ms = ctypes.c_float()
        self._check(_lib.vkc_timer_stop(self.handle, ctypes.byref(ms)))
        return ms.value

    @property
    def stream(self):
        return _lib.vkc_get_stream(self.handle)

    # ---------------------------------------------------------------- batches and graphs

    def batch(self, arrays):
        return Batch(self, arrays)

    def batch_filter_sum(self, batch, cmp, c, sums):
        """sums[i] = reduce_add_f64(filter_<cmp>_f64(batch[i], c)) for every array (enqueued)."""
        self._check(_lib.vkc_batch_filter_sum_f64(self.handle, batch.handle, CMPS.index(cmp), c, sums.handle))

    def batch_count(self, batch, cmp, c, counts):
        """counts[i] = length(filter_<cmp>_f64(batch[i], c)) for every array (enqueued)."""
        self._check(_lib.vkc_batch_count_f64(self.handle, batch.handle, CMPS.index(cmp), c, counts.handle))

    def batch_dot(self, xs, ys, sums):
        """sums[i] = dot_f64(xs[i], ys[i]) for every pair (enqueued)."""
        self._check(_lib.vkc_batch_dot_f64(self.handle, xs.handle, ys.handle, sums.handle))

    def batch_argsort(self, keys, outs, key_digits=0):
        """outs[i] = argsort_i64(keys[i]) for every array (enqueued)."""
        self._check(_lib.vkc_batch_argsort_i64(self.handle, keys.handle, outs.handle, key_digits))

    def batch_rand(self, type_name, lens, seeds):
        """rand_f64 / rand_i64 (type_name "f64" or "i64") of every (len, seed) pair, one launch."""
        k = len(lens)
        ln = (ctypes.c_int64 * max(1, k))(*[int(v) for v in lens])
        sd = (ctypes.c_int64 * max(1, k))(*[int(v) for v in seeds])
        outs = (_P * max(1, k))()
        self._check(_lib.vkc_batch_rand(self.handle, TYPES[type_name], k, ln, sd, outs))
        return [Array(self, outs[i]) for i in range(k)]

    def batch_concat(self, batch, index=True):
        """The batch's arrays concatenated in order, and (index=True) the i64 column naming each
        row's array: (rows, index) or rows alone."""
        r, ix = _P(), _P()
        self._check(_lib.vkc_batch_concat(self.handle, batch.handle, ctypes.byref(r),
                                          ctypes.byref(ix) if index else None))
        rows = Array(self, r.value)
        return (rows, Array(self, ix.value)) if index else rows

    def graph_begin(self):
        self._check(_lib.vkc_graph_begin(self.handle))

    def graph_end(self):
        h = _P()
        self._check(_lib.vkc_graph_end(self.handle, ctypes.byref(h)))
        return Graph(self, h.value)


class Reducer:
    """Dispatch::reducer: tile-fed reduction state (every update but the last has a multiple
    of 16 rows)."""

    def __init__(self, ctx, name):
        self.ctx = ctx
        h = _P()
        ctx._check(_lib.vkc_reducer_new(ctx.handle, ctx.kernel_id(name), ctypes.byref(h)))
        self.handle = h.value

    def update(self, *args):
        vals = self.ctx._values(args)
        self.ctx._check(_lib.vkc_reducer_update(self.handle, vals, len(args)))

    def finish(self, raw=False):
        s = _Scalar()
        h, self.handle = self.handle, None
        self.ctx._check(_lib.vkc_reducer_finish(h, ctypes.byref(s)))
        return _scalar_bits_value(s) if raw else _scalar_from_c(s)

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.vkc_reducer_free(self.handle)


class Scanner:
    """Dispatch::scanner: tile-fed scan state."""

    def __init__(self, ctx, name):
        self.ctx = ctx
        h = _P()
        ctx._check(_lib.vkc_scanner_new(ctx.handle, ctx.kernel_id(name), ctypes.byref(h)))
        self.handle = h.value

    def update(self, args, out):
        vals = self.ctx._values(args)
        self.ctx._check(_lib.vkc_scanner_update(self.handle, vals, len(args), out.handle))

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.vkc_scanner_free(self.handle)


class Builder:
    """ArrayBuilder on the device, for select_tile."""

    def __init__(self, ctx, type_name):
        self.ctx = ctx
        h = _P()
        ctx._check(_lib.vkc_builder_new(ctx.handle, TYPES[type_name], ctypes.byref(h)))
        self.handle = h.value

    def finish(self):
        h = _P()
        b, self.handle = self.handle, None
        self.ctx._check(_lib.vkc_builder_finish(b, ctypes.byref(h)))
        return Array(self.ctx, h.value)

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.vkc_builder_free(self.handle)


CMPS = ["eq", "ne", "lt", "le", "gt", "ge"]


class Batch:
    """Many arrays of one type that run the same statement (vkc_batch); keeps them alive."""

    def __init__(self, ctx, arrays):
        self.ctx = ctx
        self.arrays = list(arrays)
        handles = (_P * max(1, len(self.arrays)))(*[a.handle for a in self.arrays])
        h = _P()
        ctx._check(_lib.vkc_batch_new(ctx.handle, len(self.arrays), handles, ctypes.byref(h)))
        self.handle = h.value

    def __len__(self):
        return len(self.arrays)

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.vkc_batch_free(self.handle)


class Graph:
    """A captured CUDA graph of enqueued library work (vkc_graph)."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle

    def launch(self):
        self.ctx._check(_lib.vkc_graph_launch(self.ctx.handle, self.handle))

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.vkc_graph_free(self.handle)
