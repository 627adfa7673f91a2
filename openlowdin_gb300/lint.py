"""ctypes binding of liblowdin_gb300.so.

`Libint2Interface` mirrors the Fortran module src/ints/Libint2Interface.f90 of
openLOWDIN: one object per species, built from the species' shells in basis
order (Libint2Interface_constructor, :382-448), with the direct two-particle,
coupling and first-quarter calls (:514-707).  Every call goes through the C ABI
declared in include/lowdin_gb300.h -- the same entry points a Fortran
ISO_C_BINDING interface binds.

Host-buffer calls (`compute_2body_direct`, ...) behave like the reference: they
take and return numpy arrays and synchronise.  Device calls
(`twobody_device`, `coupling_device`) take raw device pointers (e.g.
torch.Tensor.data_ptr()) and a CUDA stream handle and queue work only.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblowdin_gb300.so")
_LIB = None

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p


# shell-pair classes of the library (s, p, d, f shells: ss ps pp ds dp dd fs fp fd ff),
# the index of class (la >= lb) being la (la + 1) / 2 + lb
NPC = 10
PAIR_CLASSES = [(la, lb) for la in range(4) for lb in range(la + 1)]


class LowdinGB300Error(RuntimeError):
    pass


def lib():
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise LowdinGB300Error(
                f"{LIB_PATH} is missing: build it with `python -m openlowdin_gb300.build` "
                "(nvcc, sm_103a). There is no CPU fallback.")
        L = ctypes.CDLL(LIB_PATH)
        L.LibintInterface_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_bool, ctypes.c_bool]
        L.LibintInterface_new.restype = _vp
        L.LibintInterface_del.argtypes = [_vp]
        L.LibintInterface_add_particle.argtypes = [_vp, ctypes.c_int, _f64p]
        L.LibintInterface_add_shell.argtypes = [_vp, _f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_int]
        L.LibintInterface_get_nbasis.argtypes = [_vp]
        L.LibintInterface_get_nbasis.restype = ctypes.c_int
        L.LibintInterface_compute_1body_ints.argtypes = [_vp, ctypes.c_int, _f64p]
        L.LibintInterface_init_2body_ints.argtypes = [_vp]
        L.LibintInterface_compute_2body_direct.argtypes = [_vp, _f64p, _f64p, ctypes.POINTER(ctypes.c_double)]
        L.LibintInterface_compute_2body_directIT.argtypes = [_vp, _f64p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int)]
        L.LibintInterface_compute_coupling_direct.argtypes = [_vp, _vp, _f64p, _f64p]
        L.LibintInterface_compute_alphabeta_direct.argtypes = [_vp, _vp, _f64p, _f64p, _f64p]
        L.LowdinGB300_set_precision.argtypes = [_vp, ctypes.c_int, ctypes.c_double]
        L.LowdinGB300_set_precision.restype = ctypes.c_int
        L.libintinterface_compute_g12_direct.argtypes = [_vp, _f64p, _f64p, ctypes.POINTER(ctypes.c_double),
                                                         _f64p, _f64p, ctypes.c_int]
        L.libintinterface_compute_g12inter_direct.argtypes = [_vp, _vp, _f64p, _f64p, _f64p, _f64p, ctypes.c_int]
        L.LibintInterface_compute_coupling_directIT.argtypes = [_vp, _vp, _f64p, _f64p, _f64p,
                                                                ctypes.POINTER(ctypes.c_int)]
        L.LowdinGB300_last_error.restype = ctypes.c_char_p
        L.LowdinGB300_potential.argtypes = [_vp, ctypes.c_int, _f64p, _f64p, _f64p]
        L.LowdinGB300_gaussian_potential.argtypes = [_vp, ctypes.c_int, _f64p, _f64p, _f64p, _f64p]
        L.LowdinGB300_twobody_device.argtypes = [_vp, _vp, _vp, ctypes.c_double, ctypes.c_int, ctypes.c_double, _vp]
        L.LowdinGB300_twobody_device.restype = ctypes.c_int
        L.LowdinGB300_one_body_device.argtypes = [_vp, ctypes.c_int, _f64p, _f64p, _vp, _vp, _vp, _vp]
        L.LowdinGB300_one_body_device.restype = ctypes.c_int
        L.LowdinGB300_coupling_device.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]
        L.LowdinGB300_coupling_device.restype = ctypes.c_int
        L.LowdinGB300_last_quartets.argtypes = [_vp]
        L.LowdinGB300_last_quartets.restype = ctypes.c_longlong
        L.LowdinGB300_version.restype = ctypes.c_char_p
        L.LowdinGB300_last_class_quartets.argtypes = [_vp, np.ctypeslib.ndpointer(dtype=np.int64)]
        L.LowdinGB300_last_class_quartets.restype = ctypes.c_int
        L.LowdinGB300_pair_class_counts.argtypes = [_vp, ctypes.c_int, np.ctypeslib.ndpointer(dtype=np.int32)]
        L.LowdinGB300_pair_class_counts.restype = ctypes.c_int
        L.LowdinGB300_measure_fma_tflops.argtypes = [ctypes.c_int]
        L.LowdinGB300_measure_fma_tflops.restype = ctypes.c_double
        L.LowdinGB300_launch_count.restype = ctypes.c_longlong
        L.LowdinGB300_noalloc_scratch_bytes.restype = ctypes.c_size_t
        L.LowdinGB300_twobody_device_noalloc.argtypes = [_vp, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                                         ctypes.c_double, _vp]
        L.LowdinGB300_twobody_device_noalloc.restype = ctypes.c_int
        L.LowdinGB300_mp2_direct.argtypes = [_vp, _vp, _vp, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.POINTER(ctypes.c_double), _vp]
        L.LowdinGB300_mp2_direct.restype = ctypes.c_int
        L.LowdinGB300_mp2_last_columns.restype = ctypes.c_longlong
        L.LowdinGB300_mp2_moint.argtypes = [_vp, _vp, _vp, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                            ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_longlong), _vp]
        L.LowdinGB300_mp2_moint.restype = ctypes.c_int
        L.LowdinGB300_mp2_coupling_moint.argtypes = [_vp, _vp, _vp, _vp, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                                     ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                                     ctypes.POINTER(ctypes.c_longlong), _vp]
        L.LowdinGB300_mp2_coupling_moint.restype = ctypes.c_int
        _i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.LowdinGB300_moint_write.argtypes = [ctypes.c_char_p, ctypes.c_int, _i32p, _i32p, _i32p, _i32p, _f64p,
                                              ctypes.c_longlong]
        L.LowdinGB300_moint_write.restype = ctypes.c_int
        L.LowdinGB300_mp2_coupling.argtypes = [_vp, _vp, _vp, _vp, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                               ctypes.c_double, ctypes.POINTER(ctypes.c_double), _vp]
        L.LowdinGB300_mp2_coupling.restype = ctypes.c_int
        L.LowdinGB300_diis_coefficients.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]
        L.LowdinGB300_diis_coefficients.restype = ctypes.c_int
        L.LowdinGB300_batch_autotune.argtypes = [_vp, ctypes.c_double, ctypes.c_int, _vp]
        L.LowdinGB300_batch_autotune.restype = ctypes.c_int
        L.LowdinGB300_batch_tuning.argtypes = [_vp, np.ctypeslib.ndpointer(dtype=np.int32),
                                               np.ctypeslib.ndpointer(dtype=np.float32),
                                               np.ctypeslib.ndpointer(dtype=np.float32)]
        L.LowdinGB300_batch_tuning.restype = ctypes.c_int
        L.LowdinGB300_boys_eval.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, _f64p]
        L.LowdinGB300_boys_eval.restype = ctypes.c_int
        L.LowdinGB300_gemm_bf16_split.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_int, _vp]
        L.LowdinGB300_gemm_bf16_split.restype = ctypes.c_int
        L.LowdinGB300_gemm_bf16_precise.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp]
        L.LowdinGB300_gemm_bf16_precise.restype = ctypes.c_int
        L.LowdinGB300_gemm_bench.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             _vp]
        L.LowdinGB300_gemm_bench.restype = ctypes.c_double
        L.LowdinGB300_batch_new.restype = _vp
        L.LowdinGB300_batch_del.argtypes = [_vp]
        L.LowdinGB300_batch_add_system.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.c_int, _f64p, _f64p,
                                                   np.ctypeslib.ndpointer(dtype=np.int32), ctypes.POINTER(_vp),
                                                   ctypes.POINTER(_vp), ctypes.POINTER(_vp)]
        L.LowdinGB300_batch_add_system.restype = ctypes.c_int
        L.LowdinGB300_batch_add_system_ld.argtypes = L.LowdinGB300_batch_add_system.argtypes + [
            np.ctypeslib.ndpointer(dtype=np.int32)]
        L.LowdinGB300_batch_add_system_ld.restype = ctypes.c_int
        L.LowdinGB300_batch_set_skip.argtypes = [_vp, ctypes.c_double]
        L.LowdinGB300_batch_set_skip.restype = ctypes.c_int
        L.LowdinGB300_batch_set_active.argtypes = [_vp, np.ctypeslib.ndpointer(dtype=np.int32), _vp]
        L.LowdinGB300_batch_set_active.restype = ctypes.c_int
        L.LowdinGB300_batch_finalize.argtypes = [_vp, _vp]
        L.LowdinGB300_batch_finalize.restype = ctypes.c_int
        L.LowdinGB300_batch_fock.argtypes = [_vp, ctypes.c_int, ctypes.c_double, _vp]
        L.LowdinGB300_batch_fock.restype = ctypes.c_int
        L.LowdinGB300_batch_use_graph.argtypes = [_vp, ctypes.c_int]
        L.LowdinGB300_batch_use_graph.restype = ctypes.c_int
        L.LowdinGB300_batch_quartets.argtypes = [_vp, np.ctypeslib.ndpointer(dtype=np.int64), _vp]
        L.LowdinGB300_batch_quartets.restype = ctypes.c_int
        L.LowdinGB300_batch_coupling_quartets.argtypes = [_vp, np.ctypeslib.ndpointer(dtype=np.int64), _vp]
        L.LowdinGB300_batch_coupling_quartets.restype = ctypes.c_int
        _LIB = L
    return _LIB


# every symbol include/lowdin_gb300.h declares
EXPORTED_SYMBOLS = [
    "LibintInterface_new", "LibintInterface_del", "LibintInterface_add_particle", "LibintInterface_add_shell",
    "LibintInterface_get_nbasis", "LibintInterface_compute_1body_ints", "LibintInterface_init_2body_ints",
    "LibintInterface_compute_2body_direct", "LibintInterface_compute_2body_directIT",
    "LibintInterface_compute_2body_disk", "LibintInterface_compute_coupling_direct",
    "LibintInterface_compute_coupling_directIT", "LibintInterface_compute_alphabeta_direct",
    "LibintInterface_compute_coupling_disk", "libintinterface_compute_g12_disk",
    "libintinterface_compute_g12inter_disk", "libintinterface_compute_g12_direct",
    "libintinterface_compute_g12inter_direct", "LibintInterface_compute_2body_directAll",
    "LibintInterface_compute_coupling_directAll", "libintinterface_compute_g12_directAll",
    "libintinterface_compute_g12inter_directAll", "LowdinGB300_last_error", "LowdinGB300_clear_error",
    "LowdinGB300_potential", "LowdinGB300_gaussian_potential", "LowdinGB300_set_precision", "LowdinGB300_twobody_device", "LowdinGB300_one_body_device", "LowdinGB300_coupling_device",
    "LowdinGB300_last_quartets", "LowdinGB300_version", "LowdinGB300_last_class_quartets",
    "LowdinGB300_pair_class_counts", "LowdinGB300_measure_fma_tflops", "LowdinGB300_launch_count",
    "LowdinGB300_batch_new", "LowdinGB300_batch_del", "LowdinGB300_batch_add_system",
    "LowdinGB300_batch_add_system_ld", "LowdinGB300_batch_set_active", "LowdinGB300_batch_set_skip",
    "LowdinGB300_batch_finalize", "LowdinGB300_batch_fock", "LowdinGB300_batch_use_graph",
    "LowdinGB300_batch_quartets",
    "LowdinGB300_batch_coupling_quartets", "LowdinGB300_noalloc_scratch_bytes",
    "LowdinGB300_twobody_device_noalloc", "LowdinGB300_mp2_direct", "LowdinGB300_mp2_last_columns", "LowdinGB300_mp2_coupling",
    "LowdinGB300_gemm_bf16_split", "LowdinGB300_gemm_bf16_precise",
    "LowdinGB300_gemm_bench", "LowdinGB300_mp2_moint", "LowdinGB300_mp2_coupling_moint", "LowdinGB300_moint_write",
    "LowdinGB300_diis_coefficients", "LowdinGB300_boys_eval", "LowdinGB300_batch_autotune",
    "LowdinGB300_batch_tuning",
]


def diis_coefficients(e_ptr: int, h: int, nsys: int, coef_ptr: int, stream: int = 0, first_ptr: int = 0):
    """DIIS coefficients of nsys systems from their [h][h] error products
    (device FP64 arrays), queued on `stream`; first_ptr: optional device int
    array, per system the first history entry used."""
    if lib().LowdinGB300_diis_coefficients(e_ptr, h, nsys, first_ptr or None, coef_ptr, stream) != 0:
        _check()


def boys_eval(T, L: int, fp32: bool) -> np.ndarray:
    """F_0..F_L at the arguments T from the device Boys function of the FP32
    (fp32) or FP64 kernels; shape [len(T), L + 1]."""
    T = np.ascontiguousarray(T, dtype=np.float64)
    out = np.zeros((len(T), L + 1))
    if lib().LowdinGB300_boys_eval(1 if fp32 else 0, L, T, len(T), out) != 0:
        _check()
    return out


def moint_write(path: str, p, q, r, s, v, stack_size: int = 30000):
    """Entries (1-based orbital numbers p, q, r, s and values v, in order) to a
    moint.dat-layout file (LowdinGB300_moint_write; host only)."""
    a = [np.ascontiguousarray(x, np.int32) for x in (p, q, r, s)]
    vv = np.ascontiguousarray(v, np.float64)
    if lib().LowdinGB300_moint_write(os.fsencode(path), int(stack_size), *a, vv, len(vv)) != 0:
        _check()
        raise LowdinGB300Error("moint_write failed")


class Batch:
    """Many systems' two-particle + coupling builds in one set of launches.

    add_system(handles, charges, factors, two_body, P, G, J[, ld]) takes torch
    tensors (or raw device pointers) for each species' density / outputs; ld
    gives each species' row stride when its matrices sit in a larger padded
    array.  set_active(flags) switches systems' integral work off and on."""

    def __init__(self):
        self.h = lib().LowdinGB300_batch_new()
        self._keep = []

    def add_system(self, handles, charges, factors, two_body, P, G, J, ld=None) -> int:
        ns = len(handles)
        ptr = lambda x: x if isinstance(x, int) else (0 if x is None else x.data_ptr())
        hs = (_vp * ns)(*[h.h for h in handles])
        pP = (_vp * ns)(*[ptr(x) for x in P])
        pG = (_vp * ns)(*[ptr(x) for x in G])
        pJ = (_vp * ns)(*[ptr(x) for x in J])
        self._keep.append((handles, P, G, J))
        args = (self.h, hs, ns, np.ascontiguousarray(charges, np.float64),
                np.ascontiguousarray(factors, np.float64), np.ascontiguousarray(two_body, np.int32), pP, pG, pJ)
        if ld is None:
            k = lib().LowdinGB300_batch_add_system(*args)
        else:
            k = lib().LowdinGB300_batch_add_system_ld(*args, np.ascontiguousarray(ld, np.int32))
        if k < 0:
            _check()
            raise LowdinGB300Error("batch add_system failed")
        self.nsys = getattr(self, "nsys", 0) + 1
        return k

    def set_skip(self, skip: float):
        """Mixed builds drop quartets whose density-weighted bound is below skip."""
        if lib().LowdinGB300_batch_set_skip(self.h, float(skip)) != 0:
            raise LowdinGB300Error(f"batch set_skip({skip}) failed")

    def set_active(self, flags, stream: int = 0):
        """flags[s] (in add order): 0 = system s is not built by the next fock
        calls, 1 = built, 2 = built with every quartet in FP64 in mixed builds."""
        f = np.clip(np.ascontiguousarray(np.asarray(flags).astype(np.int64), np.int32), 0, 2).astype(np.int32)
        if f.size != getattr(self, "nsys", 0):
            raise ValueError(f"set_active wants {getattr(self, 'nsys', 0)} flags, got {f.size}")
        self._flags = f
        if lib().LowdinGB300_batch_set_active(self.h, f, stream) != 0:
            _check()
            raise LowdinGB300Error("batch set_active failed")

    def finalize(self, stream: int = 0):
        if lib().LowdinGB300_batch_finalize(self.h, stream) != 0:
            _check()
            raise LowdinGB300Error("batch finalize failed")

    def autotune(self, split: float = 1e-5, force: bool = False, stream: int = 0):
        """Pick the faster FP32 kernel per quartet class for mixed builds
        (LowdinGB300_batch_autotune)."""
        if lib().LowdinGB300_batch_autotune(self.h, float(split), int(bool(force)), stream) != 0:
            _check()
            raise LowdinGB300Error("batch autotune failed")

    def tuning(self):
        """(choice [6, 6], ms bra-row kernel [6, 6], ms one-quartet-per-thread
        kernel [6, 6]) of the last autotune."""
        ch = np.zeros(NPC * NPC, np.int32)
        a = np.zeros(NPC * NPC, np.float32)
        b = np.zeros(NPC * NPC, np.float32)
        lib().LowdinGB300_batch_tuning(self.h, ch, a, b)
        return ch.reshape(NPC, NPC), a.reshape(NPC, NPC), b.reshape(NPC, NPC)

    def use_graph(self, on: bool):
        lib().LowdinGB300_batch_use_graph(self.h, int(bool(on)))

    def fock(self, precision: int = 0, split: float = 0.0, stream: int = 0):
        if lib().LowdinGB300_batch_fock(self.h, int(precision), float(split), stream) != 0:
            _check()
            raise LowdinGB300Error("batch fock failed")

    def quartets(self, stream: int = 0) -> np.ndarray:
        out = np.zeros(NPC * NPC, np.int64)
        if lib().LowdinGB300_batch_quartets(self.h, out, stream) < 0:
            _check()
        return out.reshape(NPC, NPC)

    def coupling_quartets(self, stream: int = 0) -> np.ndarray:
        out = np.zeros(NPC * NPC, np.int64)
        if lib().LowdinGB300_batch_coupling_quartets(self.h, out, stream) < 0:
            _check()
        return out.reshape(NPC, NPC)

    def close(self):
        if getattr(self, "h", None):
            lib().LowdinGB300_batch_del(self.h)
            self.h = None
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().LowdinGB300_launch_count())


def last_error() -> str:
    return lib().LowdinGB300_last_error().decode()


def _check():
    err = last_error()
    if err:
        lib().LowdinGB300_clear_error()
        raise LowdinGB300Error(err)


class Libint2Interface:
    """One species' handle (the reference's Libint2Instance(speciesID))."""

    def __init__(self, species: dict, species_id: int, stack_size: int = 30000):
        L = lib()
        self.species = species
        self.species_id = int(species_id)
        self.is_electron = bool(species.get("is_electron", False))
        self.h = L.LibintInterface_new(int(stack_size), self.species_id, self.is_electron, True)
        for l, alphas, coefs, origin in species["shells"]:
            a = np.ascontiguousarray(alphas, np.float64)
            c = np.ascontiguousarray(coefs, np.float64)
            o = np.ascontiguousarray(origin, np.float64)
            L.LibintInterface_add_shell(self.h, a, c, o, int(l), len(a))
        self.nbasis = L.LibintInterface_get_nbasis(self.h)
        _check()

    def close(self):
        if getattr(self, "h", None):
            lib().LibintInterface_del(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------- host-buffer calls --
    def init_2body_ints(self):
        lib().LibintInterface_init_2body_ints(self.h)
        _check()

    def compute_2body_direct(self, density: np.ndarray, factor: float) -> np.ndarray:
        """Libint2Interface_compute2BodyIntraspecies_direct (before the q^2 scaling)."""
        n = self.nbasis
        D = np.ascontiguousarray(density, np.float64)
        out = np.empty((n, n))
        f = ctypes.c_double(factor)
        lib().LibintInterface_compute_2body_direct(self.h, D, out, ctypes.byref(f))
        _check()
        return out

    def compute_coupling_direct(self, other: "Libint2Interface", other_density: np.ndarray) -> np.ndarray:
        """Libint2Interface_compute2BodyInterspecies_direct: lower triangle (row >= col)."""
        n = self.nbasis
        out = np.empty((n, n))
        lib().LibintInterface_compute_coupling_direct(self.h, other.h, np.ascontiguousarray(other_density, np.float64),
                                                      out)
        _check()
        return out

    def compute_alphabeta_direct(self, other: "Libint2Interface", density, other_density) -> float:
        """Libint2Interface_compute2BodyAlphaBeta_direct: sum D (ij|kl) D_other."""
        out = np.zeros(1)
        lib().LibintInterface_compute_alphabeta_direct(self.h, other.h, np.ascontiguousarray(density, np.float64),
                                                       np.ascontiguousarray(other_density, np.float64), out)
        _check()
        return float(out[0])

    def set_precision(self, precision: int, split: float = 1e-5):
        """Precision of compute_2body_direct: 0 FP64, 1 FP32/FP64 split at `split`."""
        if lib().LowdinGB300_set_precision(self.h, int(precision), float(split)) != 0:
            _check()

    def compute_g12_direct(self, density, factor: float, coefficients, exponents) -> np.ndarray:
        """Libint2Interface_computeG12Intraspecies_direct: the two-particle matrix of
        the potential sum_k c_k exp(-g_k r12^2) (coefficients c_k, exponents g_k)."""
        n = self.nbasis
        c = np.ascontiguousarray(coefficients, np.float64).ravel()
        g = np.ascontiguousarray(exponents, np.float64).ravel()
        if c.shape != g.shape:
            raise ValueError("geminal coefficients and exponents differ in length")
        out = np.empty((n, n))
        f = ctypes.c_double(factor)
        lib().libintinterface_compute_g12_direct(self.h, np.ascontiguousarray(density, np.float64), out,
                                                 ctypes.byref(f), c, g, len(c))
        _check()
        return out

    def compute_g12inter_direct(self, other: "Libint2Interface", other_density, coefficients,
                                exponents) -> np.ndarray:
        """Libint2Interface_computeG12Interspecies_direct: lower triangle (row >= col)."""
        n = self.nbasis
        c = np.ascontiguousarray(coefficients, np.float64).ravel()
        g = np.ascontiguousarray(exponents, np.float64).ravel()
        if c.shape != g.shape:
            raise ValueError("geminal coefficients and exponents differ in length")
        out = np.empty((n, n))
        lib().libintinterface_compute_g12inter_direct(self.h, other.h, np.ascontiguousarray(other_density, np.float64),
                                                      out, c, g, len(c))
        _check()
        return out

    def compute_2body_directIT(self, density, coefficients, p: int) -> np.ndarray:
        n = self.nbasis
        out = np.empty(n * n * n)
        pp = ctypes.c_int(p)
        lib().LibintInterface_compute_2body_directIT(self.h, np.ascontiguousarray(density, np.float64),
                                                     np.ascontiguousarray(coefficients, np.float64), out,
                                                     ctypes.byref(pp))
        _check()
        return out.reshape(n, n, n)

    def compute_coupling_directIT(self, other: "Libint2Interface", coefficients, p: int) -> np.ndarray:
        n, on = self.nbasis, other.nbasis
        out = np.empty(n * on * on)
        pp = ctypes.c_int(p)
        dummy = np.zeros((n, n))
        lib().LibintInterface_compute_coupling_directIT(self.h, other.h, dummy,
                                                        np.ascontiguousarray(coefficients, np.float64), out,
                                                        ctypes.byref(pp))
        _check()
        return out.reshape(n, on, on)

    def one_body(self, kind: int) -> np.ndarray:
        n = self.nbasis
        out = np.empty((n, n))
        lib().LibintInterface_compute_1body_ints(self.h, int(kind), out)
        _check()
        return out

    def potential(self, charges, positions) -> np.ndarray:
        n = self.nbasis
        out = np.empty((n, n))
        Z = np.ascontiguousarray(charges, np.float64)
        R = np.ascontiguousarray(positions, np.float64).reshape(-1)
        lib().LowdinGB300_potential(self.h, len(Z), Z, R if len(R) else np.zeros(3), out)
        _check()
        return out

    def gaussian_potential(self, coefficients, exponents, origins) -> np.ndarray:
        """External Gaussian-fit potential sum_k c_k <i|exp(-g_k |r - C_k|^2)|j>
        (host, LowdinGB300_gaussian_potential)."""
        n = self.nbasis
        out = np.empty((n, n))
        c = np.ascontiguousarray(coefficients, np.float64)
        g = np.ascontiguousarray(exponents, np.float64)
        C = np.ascontiguousarray(origins, np.float64).reshape(-1)
        if len(c) != len(g) or len(C) != 3 * len(c):
            raise ValueError("gaussian_potential: coefficients, exponents and origins differ in length")
        lib().LowdinGB300_gaussian_potential(self.h, len(c), c if len(c) else np.zeros(1),
                                             g if len(g) else np.zeros(1), C if len(C) else np.zeros(3), out)
        _check()
        return out

    # -------------------------------------------------------- device calls --
    def one_body_device(self, charges, positions, s_ptr: int = 0, t_ptr: int = 0, v_ptr: int = 0,
                        stream: int = 0):
        """S, T and point-charge V on the device (pointers to n x n FP64, 0 to skip)."""
        Z = np.ascontiguousarray(charges, np.float64)
        R = np.ascontiguousarray(positions, np.float64).reshape(-1)
        if lib().LowdinGB300_one_body_device(self.h, len(Z), Z if len(Z) else np.zeros(1),
                                             R if len(R) else np.zeros(3), s_ptr or None, t_ptr or None,
                                             v_ptr or None, stream) != 0:
            _check()
            raise LowdinGB300Error("one_body_device failed")

    def twobody_device(self, d_ptr: int, g_ptr: int, factor: float, precision: int = 0, split: float = 0.0,
                       stream: int = 0):
        rc = lib().LowdinGB300_twobody_device(self.h, d_ptr, g_ptr, float(factor), int(precision), float(split),
                                              stream)
        if rc != 0:
            _check()
            raise LowdinGB300Error("twobody_device failed")

    def last_quartets(self) -> int:
        return int(lib().LowdinGB300_last_quartets(self.h))

    def last_class_quartets(self) -> np.ndarray:
        """[NPC][NPC] quartets per (bra pair class, ket pair class) of the last build."""
        out = np.zeros(NPC * NPC, np.int64)
        lib().LowdinGB300_last_class_quartets(self.h, out)
        return out.reshape(NPC, NPC)

    def mp2_direct(self, d_ptr: int, c_ptr: int, eps, n_occ: int, n_frozen: int = 0, precision: int = 0,
                   x_budget_gb: float = 0.0, stream: int = 0) -> float:
        """E_MP2 (closed shell) with the transform on the device; d_ptr / c_ptr:
        device n x n density and coefficients (row p = orbital p)."""
        e2 = ctypes.c_double(0.0)
        rc = lib().LowdinGB300_mp2_direct(self.h, d_ptr, c_ptr, np.ascontiguousarray(eps, np.float64),
                                          int(n_occ), int(n_frozen), int(precision), float(x_budget_gb),
                                          ctypes.byref(e2), stream)
        if rc != 0:
            _check()
            raise LowdinGB300Error("mp2_direct failed")
        return e2.value

    def mp2_moint(self, d_ptr: int, c_ptr: int, eps, n_occ: int, n_frozen: int, path: str,
                  stack_size: int = 30000, x_budget_gb: float = 0.0, stream: int = 0):
        """FP64 E_MP2 as mp2_direct, also writing every (ia|jb) to `path` in the
        reference's moint.dat layout; returns (E_MP2, integrals written)."""
        e2 = ctypes.c_double(0.0)
        nw = ctypes.c_longlong(0)
        rc = lib().LowdinGB300_mp2_moint(self.h, d_ptr, c_ptr, np.ascontiguousarray(eps, np.float64), int(n_occ),
                                         int(n_frozen), os.fsencode(path), int(stack_size), float(x_budget_gb),
                                         ctypes.byref(e2), ctypes.byref(nw), stream)
        if rc != 0:
            _check()
            raise LowdinGB300Error("mp2_moint failed")
        return e2.value, nw.value

    def mp2_coupling_moint(self, other: "Libint2Interface", ca_ptr: int, cb_ptr: int, eps_a, eps_b, n_occ_a: int,
                           n_frozen_a: int, n_occ_b: int, n_frozen_b: int, factor: float, path: str,
                           stack_size: int = 30000, x_budget_gb: float = 0.0, stream: int = 0):
        """FP64 inter-species MP2 term as mp2_coupling, also writing every
        (ia|jb) to `path` in the moint.dat layout; returns (E, integrals written)."""
        e2 = ctypes.c_double(0.0)
        nw = ctypes.c_longlong(0)
        rc = lib().LowdinGB300_mp2_coupling_moint(self.h, other.h, ca_ptr, cb_ptr,
                                                  np.ascontiguousarray(eps_a, np.float64),
                                                  np.ascontiguousarray(eps_b, np.float64), int(n_occ_a),
                                                  int(n_frozen_a), int(n_occ_b), int(n_frozen_b), float(factor),
                                                  os.fsencode(path), int(stack_size), float(x_budget_gb),
                                                  ctypes.byref(e2), ctypes.byref(nw), stream)
        if rc != 0:
            _check()
            raise LowdinGB300Error("mp2_coupling_moint failed")
        return e2.value, nw.value

    def mp2_coupling(self, other: "Libint2Interface", ca_ptr: int, cb_ptr: int, eps_a, eps_b, n_occ_a: int,
                     n_frozen_a: int, n_occ_b: int, n_frozen_b: int, factor: float, precision: int = 0,
                     x_budget_gb: float = 0.0, stream: int = 0) -> float:
        """Inter-species MP2 term of this species (A) and `other` (B)."""
        e2 = ctypes.c_double(0.0)
        rc = lib().LowdinGB300_mp2_coupling(self.h, other.h, ca_ptr, cb_ptr, np.ascontiguousarray(eps_a, np.float64),
                                            np.ascontiguousarray(eps_b, np.float64), int(n_occ_a), int(n_frozen_a),
                                            int(n_occ_b), int(n_frozen_b), float(factor), int(precision),
                                            float(x_budget_gb), ctypes.byref(e2), stream)
        if rc != 0:
            _check()
            raise LowdinGB300Error("mp2_coupling failed")
        return e2.value

    def pair_class_counts(self, all_pairs: bool) -> np.ndarray:
        out = np.zeros(NPC, np.int32)
        if lib().LowdinGB300_pair_class_counts(self.h, int(all_pairs), out) < 0:
            _check()
        return out


def gemm_bf16_split(a_ptr: int, b_ptr: int, c_ptr: int, M: int, N: int, K: int, pieces: int = 3,
                    stream: int = 0):
    """C (M x N) = A (M x K) B^T (B: N x K), FP32 device arrays, split-BF16 tensor cores."""
    if lib().LowdinGB300_gemm_bf16_split(a_ptr, b_ptr, c_ptr, int(M), int(N), int(K), int(pieces), stream) != 0:
        _check()
        raise LowdinGB300Error("gemm_bf16_split failed")


def gemm_bf16_precise(a_ptr: int, b_ptr: int, c_ptr: int, M: int, N: int, K: int, stream: int = 0):
    """C = A B^T with three BF16 pieces, eight products and FP64 slab accumulation."""
    if lib().LowdinGB300_gemm_bf16_precise(a_ptr, b_ptr, c_ptr, int(M), int(N), int(K), stream) != 0:
        _check()
        raise LowdinGB300Error("gemm_bf16_precise failed")


def gemm_bench(M: int, N: int, K: int, mode: int, reps: int = 5, stream: int = 0) -> float:
    """Milliseconds per launch of a tensor-core GEMM engine (mode 2, 3 or 8)."""
    v = float(lib().LowdinGB300_gemm_bench(int(M), int(N), int(K), int(mode), int(reps), stream))
    if v < 0:
        _check()
        raise LowdinGB300Error("gemm_bench failed")
    return v


def measure_fma_tflops(fp64: bool = True) -> float:
    """Measured FMA throughput of the current GPU (TFLOP/s)."""
    v = float(lib().LowdinGB300_measure_fma_tflops(int(fp64)))
    if v < 0:
        _check()
    return v


def coupling_device(a: Libint2Interface, b: Libint2Interface, da_ptr: int, db_ptr: int, ja_ptr: int, jb_ptr: int,
                    fp32: bool = False, stream: int = 0):
    rc = lib().LowdinGB300_coupling_device(a.h, b.h, da_ptr, db_ptr, ja_ptr, jb_ptr, int(fp32), stream)
    if rc != 0:
        _check()
        raise LowdinGB300Error("coupling_device failed")
