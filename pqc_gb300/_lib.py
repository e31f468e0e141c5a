"""Loader for the in-tree native library pqc_gb300/_build/libpqcgpu.so (C ABI: include/pqcgpu.h).

There is no fallback: if the library is missing or cannot be loaded, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpqcgpu.so")

# Every symbol declared in include/pqcgpu.h with its ctypes signature (restype, argtypes).
_c = ctypes
_vp, _sz, _u8p, _int, _uint = _c.c_void_p, _c.c_size_t, _c.c_void_p, _c.c_int, _c.c_uint
SIGNATURES = {
    "pqcgpu_ctx_create": (_int, [_c.POINTER(_vp), _int, _sz]),
    "pqcgpu_ctx_destroy": (_int, [_vp]),
    "pqcgpu_ctx_set_stream": (_int, [_vp, _vp]),
    "pqcgpu_ctx_stream": (_vp, [_vp]),
    "pqcgpu_ctx_wait": (_int, [_vp]),
    "pqcgpu_ctx_launches": (_c.c_uint64, [_vp]),
    "pqcgpu_last_error": (_c.c_char_p, []),
    "pqcgpu_version": (_c.c_char_p, []),
    "pqcgpu_alg_sizes": (_int, [_int] + [_c.POINTER(_sz)] * 6),
    "pqcgpu_kem_keypair_batch": (_int, [_vp, _int, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kem_enc_batch": (_int, [_vp, _int, _sz, _u8p, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kem_dec_batch": (_int, [_vp, _int, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kem_enc_batch_noalloc": (_int, [_int, _sz, _u8p, _u8p, _u8p, _u8p, _vp]),
    "pqcgpu_frodo_enc_shared_key_batch": (_int, [_vp, _int, _sz, _u8p, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kyber_indcpa_keypair_batch": (_int, [_vp, _int, _int, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kyber_indcpa_enc_batch": (_int, [_vp, _int, _int, _sz, _u8p, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kyber_indcpa_dec_batch": (_int, [_vp, _int, _int, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope_cpapke_keypair_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope_cpapke_enc_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope_cpapke_dec_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope512_cpapke_keypair_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope512_cpapke_enc_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_newhope512_cpapke_dec_batch": (_int, [_vp, _sz, _u8p, _u8p, _u8p, _uint]),
    "pqcgpu_kem_mixed_batch": (_int, [_vp, _vp, _sz, _uint]),
    "pqcgpu_graph_capture": (_int, [_vp, _vp, _sz, _uint, _c.POINTER(_vp)]),
    "pqcgpu_graph_launch": (_int, [_vp]),
    "pqcgpu_graph_destroy": (_int, [_vp]),
    "pqcgpu_server_create": (_int, [_c.POINTER(_vp), _int, _sz, _int, _int]),
    "pqcgpu_server_submit": (_int, [_vp, _vp, _c.POINTER(_c.c_uint64)]),
    "pqcgpu_server_wait": (_int, [_vp, _c.c_uint64, _int]),
    "pqcgpu_server_drain": (_int, [_vp]),
    "pqcgpu_server_get_stats": (_int, [_vp, _vp, _int]),
    "pqcgpu_server_get_group_stats": (_int, [_vp, _int, _int, _vp]),
    "pqcgpu_server_key_release": (_int, [_vp, _c.c_uint64]),
    "pqcgpu_server_destroy": (_int, [_vp]),
    "pqcgpu_server_run_poisson": (_int, [_vp, _vp, _sz, _c.c_double, _c.c_double, _c.c_uint64, _vp]),
    "pqcgpu_set_launch_shape": (_int, [_int, _int, _int, _int]),
    "pqcgpu_get_launch_shape": (_int, [_int, _int, _c.POINTER(_int), _c.POINTER(_int)]),
    "pqcgpu_profile_enable": (_int, [_int]),
    "pqcgpu_profile_read": (_int, [_c.c_char_p, _sz]),
    "pqcgpu_profile_trace": (_int, [_c.c_char_p, _c.POINTER(_sz)]),
    "pqcgpu_set_host_pipeline": (_int, [_sz, _sz, _sz, _int]),
    "pqcgpu_get_host_pipeline": (_int, [_c.POINTER(_sz), _c.POINTER(_sz), _c.POINTER(_sz), _c.POINTER(_int)]),
    "pqcgpu_probe_peaks": (_int, [_int, _c.POINTER(_c.c_double), _c.POINTER(_c.c_double)]),
    "pqcgpu_randombytes_init": (_int, [_u8p]),
    "pqcgpu_randombytes": (_int, [_u8p, _sz]),
    "pqcgpu_randombytes_init_nist": (_int, [_u8p, _u8p]),
    "pqcgpu_nist_coins": (_int, [_int, _int, _u8p]),
}
for _alg in ("kyber512", "kyber768", "kyber1024", "newhope1024", "frodo976", "mlkem512", "mlkem768", "mlkem1024",
             "newhope512", "frodo640", "frodo1344"):
    SIGNATURES["pqcgpu_%s_crypto_kem_keypair" % _alg] = (_int, [_u8p, _u8p])
    SIGNATURES["pqcgpu_%s_crypto_kem_enc" % _alg] = (_int, [_u8p, _u8p, _u8p])
    SIGNATURES["pqcgpu_%s_crypto_kem_dec" % _alg] = (_int, [_u8p, _u8p, _u8p])



class Job(_c.Structure):
    """pqcgpu_job of include/pqcgpu.h."""
    _fields_ = [("alg", _c.c_int32), ("op", _c.c_int32), ("n", _c.c_uint64), ("in0", _c.c_void_p),
                ("in1", _c.c_void_p), ("out0", _c.c_void_p), ("out1", _c.c_void_p)]


class Request(_c.Structure):
    """pqcgpu_request of include/pqcgpu.h."""
    _fields_ = [("alg", _c.c_int32), ("op", _c.c_int32), ("key", _c.c_uint64), ("pk", _c.c_void_p),
                ("in_", _c.c_void_p), ("out0", _c.c_void_p), ("out1", _c.c_void_p), ("key_out", _c.c_void_p)]


class ServerStats(_c.Structure):
    _fields_ = [("completed", _c.c_uint64), ("batches", _c.c_uint64), ("keys_resident", _c.c_uint64),
                ("hbm_used", _c.c_size_t), ("p50_ms", _c.c_double), ("p99_ms", _c.c_double),
                ("mean_ms", _c.c_double), ("max_ms", _c.c_double)]


class MixEntry(_c.Structure):
    _fields_ = [("alg", _c.c_int32), ("op", _c.c_int32), ("weight", _c.c_double)]


class LoadReport(_c.Structure):
    _fields_ = [("offered_per_s", _c.c_double), ("achieved_per_s", _c.c_double), ("seconds", _c.c_double),
                ("submit_seconds", _c.c_double), ("p50_ms", _c.c_double), ("p99_ms", _c.c_double),
                ("mean_ms", _c.c_double), ("max_ms", _c.c_double), ("submitted", _c.c_uint64),
                ("completed", _c.c_uint64), ("batches", _c.c_uint64)]


_lib = None


def load(path=LIB_PATH):
    """Load (once) and return the ctypes library; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libpqcgpu.so is not built (%s); run __graft_entry__.build() or "
                           "python pqc_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        raise RuntimeError("pqcgpu error %d: %s" % (rc, load().pqcgpu_last_error().decode()))
    return rc
