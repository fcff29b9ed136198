"""Python binding of libgbz (include/gbz.h) with the reference's call names.

The functions mirror the reference's C++ surface for the prover hot path:
fft / pfft (utils.cpp:904, :1583), MT_commit_Blake (merkle_tree.cpp:195),
open_tree_blake (merkle_tree.cpp:320), blake3_hash (Blake3_hash.cpp:5),
Whir_Commit_initial (Whir.cpp:158), precompute_beta (utils.cpp:198),
whir_sumcheck_step1/2 (Whir.cpp:215, :223), update_betas (Whir.cpp:325),
hash_to_field (Fiat_Shamir.cpp:29), F::_random (fieldElement.cpp:119), and
the single-party prover (prove).  Like the reference they operate in place
where the reference does and return what the reference returns; unlike the
reference they raise GbzError instead of calling exit().

Field-element arrays are numpy uint64 arrays of shape (n, 2) (`real`,
`img`) or torch tensors on the GPU with the same shape and dtype
torch.uint64 / torch.int64 (device pointers are passed straight through).

There is no CPU fallback: importing this module loads libgbz.so and every
call runs on the GPU (host-side protocol helpers aside).  A missing library
raises ImportError.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbz.so")

OK, EINVAL, ENOMEM, ECUDA, ECHECK, ESMALL = range(6)
MEM_HOST, MEM_DEVICE = 0, 1
P = (1 << 61) - 1

# Every function include/gbz.h declares; tests check the library exports them.
EXPORTS = (
    "gbz_create", "gbz_destroy", "gbz_set_stream", "gbz_get_stream", "gbz_synchronize",
    "gbz_status_string", "gbz_last_error", "gbz_host_alloc", "gbz_host_free", "gbz_device_alloc",
    "gbz_device_free", "gbz_field_ops", "gbz_blake3_64", "gbz_fft", "gbz_rs_encode",
    "gbz_merkle_commit_blake", "gbz_merkle_open_blake", "gbz_whir_commit", "gbz_precompute_beta",
    "gbz_sumcheck_quadratic", "gbz_sumcheck_fold", "gbz_whir_update_betas", "gbz_hash_to_field",
    "gbz_prng_seed", "gbz_prng_next", "gbz_prng_field", "gbz_field_ops_host",
    "gbz_prove_transcript_bytes", "gbz_prove", "gbz_prove_launches", "gbz_profile_enable",
    "gbz_profile_read", "gbz_whir_update_betas_noalloc", "gbz_rs_multifold5", "gbz_lagrange_coeff",
    "gbz_encode_rows", "gbz_column_merkle", "gbz_secret_shares", "gbz_party_aggregate",
    "gbz_cosumcheck_phase1", "gbz_cosumcheck_phase2", "gbz_prove_batch", "gbz_serve", "gbz_sched_release",
    "gbz_sumcheck_round", "gbz_party_sumcheck_rounds", "gbz_party_sumcheck", "gbz_calibrate",
    "gbz_whir_aggregate_claims", "gbz_whir_aggregate_arrays", "gbz_whir_aggregate_commitments",
    "gbz_tensor_eval_vector", "gbz_pcs_sumcheck_phase3", "gbz_ntt_set_shape", "gbz_ntt_get_shape",
    "gbz_ntt_autotune", "gbz_merkle_set_fusion", "gbz_merkle_get_fusion", "gbz_merkle_autotune",
    "gbz_set_graphs", "gbz_ntt_full_twiddles", "gbz_encode_concatenated", "gbz_leader_root",
    "gbz_whir_batch_schedule", "gbz_whir_batch_open", "gbz_pcs_schedule", "gbz_pcs_commit", "gbz_pcs_free",
    "gbz_pcs_info", "gbz_pcs_commit_data", "gbz_pcs_open", "gbz_pcs_claim", "gbz_cosumcheck",
    "gbz_cosumcheck_transcript_bytes", "gbz_whir_open", "gbz_whir_open_transcript_bytes",
    "gbz_merkle_tree_from_leaves", "gbz_pcs_open_full", "gbz_pcs_open_full_bytes", "gbz_sched_set_grouping",
    "gbz_r1cs_create", "gbz_r1cs_free", "gbz_r1cs_reduce", "gbz_piop_phase1", "gbz_piop_phase1_bytes",
    "gbz_piop_phase2", "gbz_piop_phase2_bytes", "gbz_dpcs_batch_commit", "gbz_dpcs_commit", "gbz_verify_proof",
    "gbz_dpcs_open", "gbz_dpcs_open_bytes", "gbz_pcs_open_piop", "gbz_pcs_open_piop_bytes",
    "gbz_pcs_claim_piop",
)

PROF_CATEGORIES = ("ntt", "merkle", "sumcheck", "beta", "update_betas", "query", "protocol")


SC_QUADRATIC, SC_CUBIC, SC_BATCH, SC_ZEROCHECK, SC_QUADRUPLE = range(5)
FORM_VECTORS = {SC_QUADRATIC: 2, SC_CUBIC: 3, SC_BATCH: 6, SC_ZEROCHECK: 6, SC_QUADRUPLE: 4}
FORM_DEGREE = {SC_QUADRATIC: 2, SC_CUBIC: 3, SC_BATCH: 2, SC_ZEROCHECK: 3, SC_QUADRUPLE: 4}


class SchedOpts(ctypes.Structure):
    """gbz_sched_opts: slots, in-flight depth per slot, graph replay, HBM reserve."""
    _fields_ = [("lanes", ctypes.c_int), ("depth", ctypes.c_int), ("graphs", ctypes.c_int),
                ("reserve_bytes", ctypes.c_uint64)]


class PinnedArray:
    """Page-locked host memory (gbz_host_alloc) viewed as a numpy array, so
    that host<->device copies of the scheduler overlap with proving."""

    def __init__(self, shape, dtype):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.p = ctypes.c_void_p()
        st = lib.gbz_host_alloc(ctypes.byref(self.p), max(self.nbytes, 1))
        if st != OK:
            raise GbzError(st, "gbz_host_alloc failed")
        buf = (ctypes.c_uint8 * max(self.nbytes, 1)).from_address(self.p.value)
        self.array = np.frombuffer(buf, dtype=np.uint8, count=self.nbytes).view(dtype).reshape(shape)

    def __del__(self):
        if getattr(self, "p", None) and self.p.value:
            self.array = None
            lib.gbz_host_free(self.p)
            self.p = ctypes.c_void_p()


class GbzError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (_status_name(status), status, msg))
        self.status = status


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libgbz.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, u64, i32, c_int = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int
    sig = {
        "gbz_create": (c_int, [ctypes.POINTER(vp), c_int]),
        "gbz_destroy": (None, [vp]),
        "gbz_set_stream": (c_int, [vp, vp]),
        "gbz_get_stream": (vp, [vp]),
        "gbz_synchronize": (c_int, [vp]),
        "gbz_status_string": (ctypes.c_char_p, [c_int]),
        "gbz_last_error": (ctypes.c_char_p, [vp]),
        "gbz_host_alloc": (c_int, [ctypes.POINTER(vp), u64]),
        "gbz_host_free": (None, [vp]),
        "gbz_device_alloc": (c_int, [vp, ctypes.POINTER(vp), u64]),
        "gbz_device_free": (None, [vp, vp]),
        "gbz_field_ops": (c_int, [vp, vp, vp, u64, vp, vp, vp, c_int]),
        "gbz_blake3_64": (c_int, [vp, vp, vp, u64, c_int]),
        "gbz_fft": (c_int, [vp, vp, c_int, c_int, c_int]),
        "gbz_rs_encode": (c_int, [vp, vp, u64, c_int, vp, c_int]),
        "gbz_merkle_commit_blake": (c_int, [vp, vp, u64, vp, c_int]),
        "gbz_merkle_open_blake": (c_int, [vp, u64, u64, vp, ctypes.POINTER(ctypes.c_uint32)]),
        "gbz_whir_commit": (c_int, [vp, vp, u64, c_int, vp, vp, c_int]),
        "gbz_precompute_beta": (c_int, [vp, vp, c_int, vp, c_int]),
        "gbz_sumcheck_quadratic": (c_int, [vp, vp, vp, u64, vp, c_int]),
        "gbz_sumcheck_fold": (c_int, [vp, vp, u64, vp, c_int]),
        "gbz_whir_update_betas": (c_int, [vp, vp, u64, vp, c_int, u64, vp, vp, c_int]),
        "gbz_hash_to_field": (None, [vp, vp, c_int, vp]),
        "gbz_prng_seed": (None, [vp, ctypes.c_uint32]),
        "gbz_prng_next": (i32, [vp]),
        "gbz_prng_field": (None, [vp, vp]),
        "gbz_field_ops_host": (None, [vp, vp, u64, vp, vp, vp]),
        "gbz_prove_transcript_bytes": (u64, [c_int, c_int]),
        "gbz_prove": (c_int, [vp, vp, c_int, c_int, ctypes.c_uint32, vp, u64, c_int]),
        "gbz_prove_launches": (c_int, [c_int, c_int]),
        "gbz_profile_enable": (c_int, [vp, c_int]),
        "gbz_profile_read": (c_int, [vp, c_int, c_int, vp, vp]),
        "gbz_whir_update_betas_noalloc": (c_int, [vp, u64, vp, c_int, u64, vp, vp, vp]),
        "gbz_rs_multifold5": (c_int, [vp, vp, u64, vp, c_int, vp, c_int]),
        "gbz_lagrange_coeff": (c_int, [vp, vp, c_int, vp, c_int]),
        "gbz_encode_rows": (c_int, [vp, vp, c_int, c_int, c_int, c_int, vp, c_int]),
        "gbz_column_merkle": (c_int, [vp, vp, c_int, c_int, c_int, vp, vp, c_int]),
        "gbz_secret_shares": (c_int, [vp, vp, u64, c_int, c_int, ctypes.c_uint32, vp, c_int]),
        "gbz_party_aggregate": (c_int, [vp, vp, c_int, u64, vp, vp, c_int]),
        "gbz_cosumcheck_phase1": (c_int, [vp, vp, vp, vp, vp, u64, c_int, vp, c_int]),
        "gbz_cosumcheck_phase2": (c_int, [vp, vp, u64, vp, c_int, vp, c_int]),
        "gbz_prove_batch": (c_int, [vp, c_int, vp, vp, vp, vp, vp, vp, c_int, vp, vp, vp]),
        "gbz_serve": (c_int, [vp, c_int, vp, vp, vp, vp, vp, vp, vp, c_int, vp, vp, vp]),
        "gbz_sched_release": (c_int, [vp, vp]),
        "gbz_sumcheck_round": (c_int, [vp, c_int, vp, u64, vp, vp, vp, c_int]),
        "gbz_party_sumcheck_rounds": (c_int, [u64, c_int, c_int]),
        "gbz_calibrate": (c_int, [vp, vp, vp]),
        "gbz_ntt_set_shape": (c_int, [c_int, c_int, c_int, c_int]),
        "gbz_ntt_get_shape": (c_int, [c_int, vp]),
        "gbz_ntt_autotune": (c_int, [vp, c_int, c_int, vp, vp, vp]),
        "gbz_merkle_set_fusion": (c_int, [c_int]),
        "gbz_set_graphs": (c_int, [vp, c_int]),
        "gbz_ntt_full_twiddles": (None, [c_int]),
        "gbz_encode_concatenated": (c_int, [vp, vp, u64, c_int, c_int, c_int, vp, vp, c_int]),
        "gbz_leader_root": (None, [vp, c_int, vp]),
        "gbz_merkle_get_fusion": (c_int, []),
        "gbz_merkle_autotune": (c_int, [vp, c_int, c_int, vp, vp, vp]),
        "gbz_tensor_eval_vector": (c_int, [vp, vp, c_int, u64, c_int, c_int, vp, c_int]),
        "gbz_pcs_sumcheck_phase3": (c_int, [vp, vp, u64, vp, c_int, vp, c_int, c_int, c_int, c_int]),
        "gbz_whir_aggregate_claims": (c_int, [vp, c_int, vp, u64, c_int, vp, vp, vp, vp, vp, vp, vp, c_int]),
        "gbz_whir_aggregate_arrays": (c_int, [vp, c_int, vp, c_int, vp, u64, vp, vp, vp, vp, vp, c_int]),
        "gbz_whir_aggregate_commitments": (c_int, [vp, c_int, vp, u64, vp, c_int, c_int, vp, vp, vp, c_int]),
        "gbz_party_sumcheck": (c_int, [vp, c_int, vp, vp, vp, u64, c_int, vp, c_int, vp, vp, vp, vp, vp, vp, c_int]),
        "gbz_whir_batch_schedule": (c_int, [c_int, vp, c_int, c_int, vp, vp, vp, vp, vp]),
        "gbz_whir_batch_open": (c_int, [vp, c_int, vp, vp, vp, vp, vp, vp, c_int, c_int, vp, vp, u64, c_int]),
        "gbz_pcs_schedule": (c_int, [c_int, u64, c_int, vp, vp, vp, vp, vp]),
        "gbz_pcs_commit": (c_int, [vp, c_int, u64, c_int, vp, vp, vp, vp, c_int, ctypes.POINTER(vp), vp, vp]),
        "gbz_pcs_free": (None, [vp]),
        "gbz_pcs_info": (c_int, [vp, vp, vp, vp, vp]),
        "gbz_pcs_commit_data": (c_int, [vp, vp, c_int, vp, vp, vp, c_int]),
        "gbz_pcs_open": (c_int, [vp, vp, vp, c_int, vp, vp, vp, u64, c_int]),
        "gbz_pcs_claim": (c_int, [vp, vp, vp, c_int, vp, c_int]),
        "gbz_cosumcheck": (c_int, [vp, c_int, c_int, u64, vp, vp, vp, vp, vp, c_int, vp, vp, vp, vp, c_int, vp, vp,
                                   vp, vp, u64, c_int]),
        "gbz_cosumcheck_transcript_bytes": (u64, [c_int, c_int, vp, c_int]),
        "gbz_whir_open": (c_int, [vp, vp, c_int, c_int, vp, vp, vp, vp, vp, u64, c_int]),
        "gbz_whir_open_transcript_bytes": (u64, [c_int, c_int]),
        "gbz_merkle_tree_from_leaves": (c_int, [vp, vp, u64, vp, c_int]),
        "gbz_pcs_open_full": (c_int, [vp, vp, vp, c_int, vp, vp, vp, vp, vp, u64, c_int]),
        "gbz_pcs_open_full_bytes": (c_int, [vp, vp]),
        "gbz_sched_set_grouping": (c_int, [vp, c_int]),
        "gbz_r1cs_create": (c_int, [vp, c_int, u64, c_int, vp, vp, vp, vp]),
        "gbz_r1cs_free": (c_int, [vp]),
        "gbz_r1cs_reduce": (c_int, [vp, vp, vp, c_int, vp, c_int, vp, vp, vp, c_int]),
        "gbz_piop_phase1": (c_int, [vp, c_int, u64, vp, vp, vp, vp, vp, vp, c_int, vp, vp, vp, vp, vp, vp, vp, u64,
                                    c_int]),
        "gbz_piop_phase1_bytes": (u64, [c_int, u64, vp, c_int]),
        "gbz_piop_phase2": (c_int, [vp, c_int, u64, vp, vp, vp, c_int, vp, vp, vp, vp, c_int, vp, c_int, vp, vp, vp,
                                    vp, vp, vp, vp, vp, vp, vp, u64, c_int]),
        "gbz_piop_phase2_bytes": (u64, [c_int, vp, c_int]),
        "gbz_dpcs_batch_commit": (c_int, [vp, c_int, u64, vp, vp, c_int, c_int, vp, vp, vp, vp, vp, c_int]),
        "gbz_dpcs_commit": (c_int, [vp, c_int, u64, vp, c_int, vp, vp, vp, vp, c_int]),
        "gbz_verify_proof": (c_int, [vp, u64, c_int, c_int, ctypes.c_uint32, vp]),
        "gbz_dpcs_open": (c_int, [vp, c_int, c_int, c_int, u64, c_int, vp, vp, vp, vp, c_int, c_int, vp, vp, vp, vp,
                                  vp, vp, vp, vp, u64, c_int]),
        "gbz_dpcs_open_bytes": (u64, [c_int, c_int, c_int]),
        "gbz_pcs_open_piop": (c_int, [vp, vp, vp, c_int, vp, u64, vp, c_int, vp, vp, c_int, vp, vp, vp, vp, vp, vp,
                                      u64, c_int]),
        "gbz_pcs_open_piop_bytes": (c_int, [vp, vp, c_int, vp, vp]),
        "gbz_pcs_claim_piop": (c_int, [vp, vp, vp, c_int, vp, u64, vp, c_int, vp, c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def _status_name(s):
    return lib.gbz_status_string(s).decode()


def _ptr(a):
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch.Tensor


def _mem(a):
    if isinstance(a, np.ndarray):
        return MEM_HOST
    return MEM_DEVICE if a.is_cuda else MEM_HOST


def fe_array(n):
    return np.zeros((n, 2), dtype=np.uint64)


def _fe(a):
    if isinstance(a, np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        return a.reshape(-1, 2)
    return a


class Context:
    """One device, one stream (gbz_ctx)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        st = lib.gbz_create(ctypes.byref(h), device)
        if st != OK:
            raise GbzError(st, "gbz_create failed")
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib.gbz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        if st != OK:
            raise GbzError(st, lib.gbz_last_error(self.h).decode())

    def synchronize(self):
        self.check(lib.gbz_synchronize(self.h))

    def set_stream(self, stream_handle):
        self.check(lib.gbz_set_stream(self.h, stream_handle))

    # ---------------------------------------------------------- primitives
    def field_ops(self, a, b):
        a, b = _fe(a), _fe(b)
        n = a.shape[0]
        outs = [fe_array(n) for _ in range(3)]
        self.check(lib.gbz_field_ops(self.h, _ptr(a), _ptr(b), n, *[_ptr(o) for o in outs], MEM_HOST))
        return outs

    def blake3_hash(self, blocks):
        """blake3_hash over count 64-byte blocks -> (count, 32) uint8."""
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 64)
        out = np.zeros((blocks.shape[0], 32), dtype=np.uint8)
        self.check(lib.gbz_blake3_64(self.h, _ptr(blocks), _ptr(out), blocks.shape[0], MEM_HOST))
        return out

    def fft(self, arr, logn, inverse):
        """fft(arr, logn, flag): in place (numpy or CUDA tensor)."""
        if isinstance(arr, np.ndarray):
            assert arr.dtype == np.uint64 and arr.flags.c_contiguous and arr.size == 2 << logn
        self.check(lib.gbz_fft(self.h, _ptr(arr), logn, int(bool(inverse)), _mem(arr)))
        return arr

    def pfft(self, arr, logn, flag=False):
        """pfft computes the forward transform whatever the flag (utils.cpp:1583-1593)."""
        if (1 << logn) // (16 * 16) <= 4:
            return self.fft(arr, logn, flag)
        return self.fft(arr, logn, False)

    def rs_encode(self, arr, rate):
        arr = _fe(arr)
        m = arr.shape[0]
        out = fe_array(m * rate)
        self.check(lib.gbz_rs_encode(self.h, _ptr(arr), m, rate, _ptr(out), MEM_HOST))
        return out

    def MT_commit_Blake(self, leafs):
        """Merkle levels as a list of (count, 32) uint8 arrays, leaves first."""
        leafs = _fe(leafs)
        N = leafs.shape[0]
        flat = np.zeros((N // 2 - 1, 32), dtype=np.uint8)
        self.check(lib.gbz_merkle_commit_blake(self.h, _ptr(leafs), N, _ptr(flat), MEM_HOST))
        return split_levels(flat, N)

    def merkle_commit_flat(self, leafs):
        leafs = _fe(leafs)
        N = leafs.shape[0]
        flat = np.zeros((N // 2 - 1, 32), dtype=np.uint8)
        self.check(lib.gbz_merkle_commit_blake(self.h, _ptr(leafs), N, _ptr(flat), MEM_HOST))
        return flat

    def Whir_Commit_initial(self, arr, rate):
        """(codeword, flat Merkle levels) of arr encoded at rate."""
        arr = _fe(arr)
        m = arr.shape[0]
        L = m * rate
        cw = fe_array(L)
        flat = np.zeros((L // 2 - 1, 32), dtype=np.uint8)
        self.check(lib.gbz_whir_commit(self.h, _ptr(arr), m, rate, _ptr(cw), _ptr(flat), MEM_HOST))
        return cw, flat

    def precompute_beta(self, r):
        r = _fe(r)
        nr = r.shape[0]
        out = fe_array(1 << nr)
        self.check(lib.gbz_precompute_beta(self.h, _ptr(r), nr, _ptr(out), MEM_HOST))
        return out

    def whir_sumcheck_step1(self, arr, b):
        """quadratic_poly (a, b, c) as a (3, 2) array."""
        arr, b = _fe(arr), _fe(b)
        out = np.zeros(6, dtype=np.uint64)
        self.check(lib.gbz_sumcheck_quadratic(self.h, _ptr(arr), _ptr(b), arr.shape[0], _ptr(out), _mem(arr)))
        return out.reshape(3, 2)

    def sumcheck_fold(self, v, r):
        """Returns the folded half (the reference resizes v to it)."""
        v = np.array(_fe(v), copy=True)
        r = np.ascontiguousarray(r, dtype=np.uint64)
        self.check(lib.gbz_sumcheck_fold(self.h, _ptr(v), v.shape[0], _ptr(r), MEM_HOST))
        return v[: v.shape[0] // 2].copy()

    def whir_sumcheck_step2(self, arr, b, c):
        return self.sumcheck_fold(arr, c), self.sumcheck_fold(b, c)

    def update_betas(self, b, queries, n, r):
        """update_betas(b, queries, n) with the drawn r; returns (b', challenges)."""
        b = np.array(_fe(b), copy=True)
        q = np.ascontiguousarray(queries, dtype=np.int32)
        r = np.ascontiguousarray(r, dtype=np.uint64)
        ch = fe_array(len(q))
        self.check(lib.gbz_whir_update_betas(self.h, _ptr(b), b.shape[0], _ptr(q), len(q), n, _ptr(r),
                                             _ptr(ch), MEM_HOST))
        return b, ch

    # ------------------------------------------------- sumcheck round forms
    def sumcheck_round(self, form, vecs, b=None, r=None):
        """Round polynomial of a form (SC_*); with r the vectors (numpy,
        C-contiguous uint64 (m, 2), or CUDA tensors) are first folded in
        place to their first halves."""
        nv = FORM_VECTORS[form]
        assert len(vecs) == nv
        vs = [_fe(v) for v in vecs]
        m = vs[0].shape[0]
        for v in vs:
            if isinstance(v, np.ndarray):
                assert v.flags.c_contiguous and v.dtype == np.uint64
        arr = (ctypes.c_void_p * nv)(*[_ptr(v) for v in vs])
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.uint64).reshape(2)
        rr = None if r is None else np.ascontiguousarray(r, dtype=np.uint64).reshape(2)
        out = fe_array(FORM_DEGREE[form] + 1)
        self.check(lib.gbz_sumcheck_round(self.h, form, ctypes.cast(arr, ctypes.c_void_p), m, _ptr(bb), _ptr(rr),
                                          _ptr(out), _mem(vs[0])))
        return out

    def party_sumcheck(self, form, vecs, N, w=None, offset=4, fs=(0, 0), prng=None, y=(0, 0)):
        """_quadratic_sumcheck / _cubic_sumcheck of N parties on this device
        (vectors of N*M entries, party-major).  Returns a dict with polys,
        challenges, fin, y, fs, prng."""
        nv = FORM_VECTORS[form]
        vs = [_fe(v) for v in vecs]
        assert len(vs) == nv
        M = vs[0].shape[0] // N
        rounds = lib.gbz_party_sumcheck_rounds(M, N, offset)
        if rounds < 0:
            raise GbzError(EINVAL, "party sumcheck: bad shape")
        nc = FORM_DEGREE[form] + 1
        polys = fe_array(max(rounds, 1) * nc)
        chal = fe_array(max(rounds, 1))
        fin = fe_array(nv)
        ww = None if w is None else np.ascontiguousarray(w, dtype=np.uint64).reshape(-1, 2)
        fsa = np.ascontiguousarray(fs, dtype=np.uint64).reshape(2).copy()
        ya = np.ascontiguousarray(y, dtype=np.uint64).reshape(2).copy()
        g = prng if isinstance(prng, Prng) else Prng(1 if prng is None else prng)
        v3 = vs[2] if nv == 3 else None
        self.check(lib.gbz_party_sumcheck(self.h, form, _ptr(vs[0]), _ptr(vs[1]), _ptr(v3), M, N, _ptr(ww), offset,
                                          _ptr(fsa), ctypes.addressof(g), _ptr(ya), _ptr(polys), _ptr(chal),
                                          _ptr(fin), _mem(vs[0])))
        return {"polys": polys[: rounds * nc].reshape(rounds, nc, 2), "challenges": chal[:rounds], "fin": fin,
                "y": ya, "fs": fsa, "prng": g}

    # ------------------------------------------------------ many proofs
    def _prove_many(self, arrivals, witnesses, logns, rates, seeds, lanes, depth, graphs, reserve, out):
        count = len(witnesses)
        assert len(logns) == count and len(rates) == count and len(seeds) == count
        mem = _mem(witnesses[0]) if count else MEM_HOST
        if out is None:
            out = [np.zeros(transcript_bytes(l, r), dtype=np.uint8) for l, r in zip(logns, rates)]
        wp = (ctypes.c_void_p * max(count, 1))(*[_ptr(_fe(w)) for w in witnesses])
        tp = (ctypes.c_void_p * max(count, 1))(*[_ptr(t) for t in out])
        cap = np.array([t.nbytes if isinstance(t, np.ndarray) else t.numel() * t.element_size() for t in out]
                       or [0], dtype=np.uint64)
        ln = np.ascontiguousarray(list(logns) or [0], dtype=np.int32)
        rt = np.ascontiguousarray(list(rates) or [0], dtype=np.int32)
        sd = np.ascontiguousarray(list(seeds) or [0], dtype=np.uint32)
        lat = np.zeros(max(count, 1), dtype=np.float64)
        mk = ctypes.c_double()
        opts = SchedOpts(lanes, depth, int(bool(graphs)), reserve)
        args = [ctypes.cast(wp, ctypes.c_void_p), _ptr(ln), _ptr(rt), _ptr(sd), ctypes.cast(tp, ctypes.c_void_p),
                _ptr(cap), mem, ctypes.byref(opts), _ptr(lat), ctypes.byref(mk)]
        if arrivals is None:
            st = lib.gbz_prove_batch(self.h, count, *args)
        else:
            arr = np.ascontiguousarray(list(arrivals) or [0.0], dtype=np.float64)
            st = lib.gbz_serve(self.h, count, _ptr(arr), *args)
        self.check(st)
        return out, lat[:count], mk.value

    def prove_batch(self, witnesses, logns, rates, seeds, lanes=8, graphs=True, reserve=0, out=None):
        """Independent proofs of mixed shapes as one batch (gbz_prove_batch).
        Returns (transcripts, per-proof completion seconds, makespan seconds)."""
        return self._prove_many(None, witnesses, logns, rates, seeds, lanes, 0, graphs, reserve, out)

    def serve(self, arrivals, witnesses, logns, rates, seeds, lanes=8, depth=2, graphs=True, reserve=0, out=None):
        """Timed arrivals (seconds from the call) through the serving loop
        (gbz_serve).  Returns (transcripts, latencies, makespan)."""
        return self._prove_many(arrivals, witnesses, logns, rates, seeds, lanes, depth, graphs, reserve, out)

    def set_grouping(self, on):
        """Whether prove_batch shares every launch among the proofs of one shape."""
        self.check(lib.gbz_sched_set_grouping(self.h, int(bool(on))))

    def sched_release(self):
        b = ctypes.c_uint64()
        self.check(lib.gbz_sched_release(self.h, ctypes.byref(b)))
        return b.value

    # ------------------------------------------------------ WHIR aggregation
    @staticmethod
    def _plist(vs):
        return ctypes.cast((ctypes.c_void_p * max(len(vs), 1))(*[_ptr(v) for v in vs]), ctypes.c_void_p)

    def aggregate_claims(self, arrays, points, prng=None):
        """aggregate_claims (Whir.cpp:608): (arr, b_aggr, K, challenges, sums)."""
        arrs = [_fe(a) for a in arrays]
        pts = np.ascontiguousarray(points, dtype=np.uint64).reshape(len(points), -1, 2)
        k, n, c = len(arrs), arrs[0].shape[0], pts.shape[0]
        arr, b = fe_array(n), fe_array(n)
        K = np.zeros(2, dtype=np.uint64)
        ch, sums = fe_array(c + k), fe_array(k * c)
        g = prng if isinstance(prng, Prng) else Prng(1 if prng is None else prng)
        self.check(lib.gbz_whir_aggregate_claims(self.h, k, self._plist(arrs), n, c, _ptr(pts), ctypes.addressof(g),
                                                 _ptr(arr), _ptr(b), _ptr(K), _ptr(ch), _ptr(sums), _mem(arrs[0])))
        return arr, b, K, ch, sums.reshape(k, c, 2), g

    def aggregate_arrays(self, arr, b, arrays, B, r1, r2):
        """aggregate_arrays (Whir.cpp:670): returns (arr', b', K)."""
        arr = np.array(_fe(arr), copy=True)
        b = np.array(_fe(b), copy=True)
        arrs, Bs = [_fe(a) for a in arrays], [_fe(x) for x in B]
        r1 = np.ascontiguousarray(r1, dtype=np.uint64).reshape(-1, 2)
        r2 = np.ascontiguousarray(r2, dtype=np.uint64).reshape(-1, 2)
        K = np.zeros(2, dtype=np.uint64)
        self.check(lib.gbz_whir_aggregate_arrays(self.h, len(arrs), self._plist(arrs), len(Bs), self._plist(Bs),
                                                 arr.shape[0], _ptr(r1), _ptr(r2), _ptr(arr), _ptr(b), _ptr(K),
                                                 MEM_HOST))
        return arr, b, K

    def whir_batch_open(self, arrays, codewords, levels0, betas, K0, rate, whir_k=4, prng=None, mem=None):
        """Whir_Batch_Open (Whir.cpp:706-898): the transcript (uint8 array, on
        the device when the inputs are torch CUDA tensors) and the advanced
        generator.  codewords[i] must have whir_batch_schedule's length for
        array i; entries of arrays that are never merged may be None."""
        k = len(arrays)
        on_dev = _mem(arrays[0]) == MEM_DEVICE if mem is None else mem == MEM_DEVICE
        conv = (lambda x: x) if on_dev else _fe
        arrs, bets = [conv(a) for a in arrays], [conv(b) for b in betas]
        sizes = np.array([int(a.shape[0]) for a in arrs], dtype=np.uint64)
        sch = whir_batch_schedule([int(x) for x in sizes], rate, whir_k)
        if sch is None:
            raise GbzError(EINVAL, "Whir_Batch_Open cannot run these sizes")
        cws = [conv(c) if c is not None else None for c in codewords]
        plist = lambda vs: ctypes.cast((ctypes.c_void_p * max(len(vs), 1))(*[_ptr(v) if v is not None else None
                                                                           for v in vs]), ctypes.c_void_p)
        lv = levels0 if on_dev else np.ascontiguousarray(levels0, dtype=np.uint8)
        K0 = np.ascontiguousarray(K0, dtype=np.uint64).reshape(2)
        g = prng if isinstance(prng, Prng) else Prng(1 if prng is None else prng)
        nbytes = sch[3]
        if on_dev:
            import torch
            out = torch.empty(nbytes, dtype=torch.uint8, device=arrays[0].device)
        else:
            out = np.zeros(nbytes, dtype=np.uint8)
        self.check(lib.gbz_whir_batch_open(self.h, k, plist(arrs), _ptr(sizes), plist(cws), _ptr(lv), plist(bets),
                                           _ptr(K0), rate, whir_k, ctypes.addressof(g), _ptr(out), nbytes,
                                           MEM_DEVICE if on_dev else MEM_HOST))
        return out, g

    def aggregate_commitments(self, codewords, r, rate, whir_k=4, prng=None):
        """aggregate_commitments (Whir.cpp:547): (codeword, levels, prng)."""
        cws = [_fe(x) for x in codewords]
        n = cws[0].shape[0]
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
        cw = fe_array(n)
        levels = np.zeros((2 * (n // whir_k) - 1, 32), dtype=np.uint8)
        g = prng if isinstance(prng, Prng) else Prng(1 if prng is None else prng)
        self.check(lib.gbz_whir_aggregate_commitments(self.h, len(cws), self._plist(cws), n, _ptr(r), rate, whir_k,
                                                      ctypes.addressof(g), _ptr(cw), _ptr(levels), MEM_HOST))
        return cw, levels, g

    def tensor_eval_vector(self, point, cols, rows, rate, my_id):
        """tensor_eval_vector (coPCS.cpp:602) for party my_id."""
        pt = np.ascontiguousarray(point, dtype=np.uint32).reshape(2)
        out = fe_array(rows)
        self.check(lib.gbz_tensor_eval_vector(self.h, _ptr(pt), cols, rows, rate, my_id, _ptr(out), MEM_HOST))
        return out

    def create_tree_blake(self, leaves):
        """create_tree_blake (merkle_tree.cpp:267) over (L, 32) leaf hashes:
        the upper levels, L/2 + ... + 1 hashes, as an (L - 1, 32) array."""
        lv = np.ascontiguousarray(leaves, dtype=np.uint8).reshape(-1, 32)
        out = np.zeros((max(lv.shape[0] - 1, 1), 32), dtype=np.uint8)
        self.check(lib.gbz_merkle_tree_from_leaves(self.h, _ptr(lv), lv.shape[0], _ptr(out), MEM_HOST))
        return out[:lv.shape[0] - 1]

    def Whir_Open(self, arr, logn, rate, codeword, point, K, prng):
        """Whir_Open (Whir.cpp:388) of the claim (K, point); prng (gbz.Prng) is
        advanced in place.  Returns the transcript bytes."""
        arr, cw = _fe(arr), _fe(codeword)
        pt = np.ascontiguousarray(point, dtype=np.uint64).reshape(-1, 2)
        Kk = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
        nb = lib.gbz_whir_open_transcript_bytes(logn, rate)
        tr = np.zeros(nb, dtype=np.uint8)
        self.check(lib.gbz_whir_open(self.h, _ptr(arr), logn, rate, _ptr(cw), _ptr(pt), _ptr(Kk),
                                     ctypes.addressof(prng), _ptr(tr), nb, MEM_HOST))
        return tr.tobytes()

    def pcs_sumcheck_phase3(self, B, queries, s, N, rate, my_id):
        """pcs_sumcheck_phase3 (coPCS.cpp:634) on a copy of B, returned."""
        B = np.array(_fe(B), copy=True)
        q = np.ascontiguousarray(queries, dtype=np.uint32).reshape(-1, 2)
        ss = np.ascontiguousarray(s, dtype=np.uint64).reshape(2)
        self.check(lib.gbz_pcs_sumcheck_phase3(self.h, _ptr(B), B.shape[0], _ptr(q), q.shape[0], _ptr(ss), N, rate,
                                               my_id, MEM_HOST))
        return B

    # ----------------------------------------------------------- coPCS side
    def RS_multifold5(self, codeword, a):
        """RS_multifold5 (coPCS_utils.cpp:386-437): fold by d = len(a)."""
        cw, a = _fe(codeword), _fe(a)
        n, d = cw.shape[0], a.shape[0]
        out = fe_array(n // d)
        self.check(lib.gbz_rs_multifold5(self.h, _ptr(cw), n, _ptr(a), d.bit_length() - 1, _ptr(out), MEM_HOST))
        return out

    def compute_lagrange_coeff(self, r, logd):
        """compute_lagrange_coeff (utils.cpp:169-197) over 2^logd points."""
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(2)
        out = fe_array(1 << logd)
        self.check(lib.gbz_lagrange_coeff(self.h, _ptr(r), logd, _ptr(out), MEM_HOST))
        return out

    def Encode(self, rows, rate, log_rate_offset):
        """Encode (coPCS.cpp:131-147) of a (rows, 2^logrow, 2) array."""
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        nrows, n = rows.shape[0], rows.shape[1]
        out = np.zeros((nrows, n * rate, 2), dtype=np.uint64)
        self.check(lib.gbz_encode_rows(self.h, _ptr(rows), nrows, n.bit_length() - 1, rate, log_rate_offset,
                                       _ptr(out), MEM_HOST))
        return out

    def encode_concatenated(self, data, rate0, rate1, degree):
        """encode_concatenated (coPCS.cpp:653): (C', C rows)."""
        data = _fe(data)
        n = data.shape[0]
        L = n * rate0
        Cp = fe_array(L)
        C = np.zeros((L // degree, degree * rate1, 2), dtype=np.uint64)
        self.check(lib.gbz_encode_concatenated(self.h, _ptr(data), n, rate0, rate1, degree, _ptr(Cp), _ptr(C),
                                               MEM_HOST))
        return Cp, C

    def distributed_MT(self, rows, nparties):
        """(levels (2L-1, 32), leader root (32,)) of one party's row batch."""
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        nrows, L = rows.shape[0], rows.shape[1]
        levels = np.zeros((2 * L - 1, 32), dtype=np.uint8)
        root = np.zeros(32, dtype=np.uint8)
        self.check(lib.gbz_column_merkle(self.h, _ptr(rows), nrows, L.bit_length() - 1, nparties, _ptr(levels),
                                         _ptr(root), MEM_HOST))
        return levels, root

    def compute_secret_shares(self, v, N, privacy=False, prng_seed=1):
        """(N, 4M/N, 2) packed Shamir shares of v (MPI_utils.cpp:2738-2764)."""
        v = _fe(v)
        M = v.shape[0]
        out = np.zeros((N, 4 * M // N, 2), dtype=np.uint64)
        self.check(lib.gbz_secret_shares(self.h, _ptr(v), M, N, int(bool(privacy)), prng_seed, _ptr(out),
                                         MEM_HOST))
        return out

    def sumcheck_aggr(self, msgs, b):
        """Leader aggregation of (N, len, 2) party messages with N/4 weights b."""
        msgs = np.ascontiguousarray(msgs, dtype=np.uint64)
        b = _fe(b)
        N, length = msgs.shape[0], msgs.shape[1]
        out = fe_array(length)
        self.check(lib.gbz_party_aggregate(self.h, _ptr(msgs), N, length, _ptr(b), _ptr(out), MEM_HOST))
        return out

    def coSumcheck_phase1(self, p1, p2, logd, p3=None, b1=None):
        """Local round sums: 2d entries (quadratic) or 4d (cubic, p3 and b1 given)."""
        p1, p2 = _fe(p1), _fe(p2)
        p3 = None if p3 is None else _fe(p3)
        b1 = None if b1 is None else _fe(b1)
        mem = _mem(p1)
        H = fe_array((4 if p3 is not None else 2) << logd)
        self.check(lib.gbz_cosumcheck_phase1(self.h, _ptr(p1), _ptr(p2), _ptr(p3), _ptr(b1), p1.shape[0], logd,
                                             _ptr(H), mem))
        return H

    def coSumcheck_phase2(self, v, L):
        """out[j] = sum_k L[k] v[j d + k] (coSumcheck.cpp:201-213)."""
        v, L = _fe(v), _fe(L)
        d = L.shape[0]
        out = fe_array(v.shape[0] // d)
        self.check(lib.gbz_cosumcheck_phase2(self.h, _ptr(v), v.shape[0], _ptr(L), d.bit_length() - 1, _ptr(out),
                                             MEM_HOST))
        return out

    # ------------------------------------------------------------ profiling
    def calibrate(self):
        """(F_{p^2} multiplies per second, Blake3 compressions per second)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        self.check(lib.gbz_calibrate(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def ntt_autotune(self, logn, reps=3):
        """Installs the fastest two-pass shape for 2^logn; returns
        (shape (k1, log_cols_a, log_rows_b), ms_default, ms_best)."""
        sh = np.zeros(3, dtype=np.int32)
        a, b = ctypes.c_double(), ctypes.c_double()
        self.check(lib.gbz_ntt_autotune(self.h, logn, reps, _ptr(sh), ctypes.byref(a), ctypes.byref(b)))
        return tuple(int(x) for x in sh), a.value, b.value

    def merkle_autotune(self, logN, reps=3):
        """Installs the faster Merkle level fusion; returns (log_nodes, ms_default, ms_best)."""
        lg = ctypes.c_int()
        a, b = ctypes.c_double(), ctypes.c_double()
        self.check(lib.gbz_merkle_autotune(self.h, logN, reps, ctypes.byref(lg), ctypes.byref(a), ctypes.byref(b)))
        return lg.value, a.value, b.value

    def set_graphs(self, on=True):
        self.check(lib.gbz_set_graphs(self.h, int(bool(on))))

    def profile_enable(self, on=True):
        self.check(lib.gbz_profile_enable(self.h, int(bool(on))))

    def profile_read(self, logn, rate):
        """{category: (milliseconds, launch groups)} since the last read."""
        ms = np.zeros(len(PROF_CATEGORIES), dtype=np.float64)
        groups = np.zeros(len(PROF_CATEGORIES), dtype=np.int32)
        self.check(lib.gbz_profile_read(self.h, logn, rate, _ptr(ms), _ptr(groups)))
        return {c: (float(ms[i]), int(groups[i])) for i, c in enumerate(PROF_CATEGORIES)}

    # --------------------------------------------------------------- prover
    def prove(self, witness, logn, rate, prng_seed=1, out=None):
        """Transcript bytes of one single-party proof (see include/gbz.h)."""
        nbytes = transcript_bytes(logn, rate)
        if nbytes == 0:
            raise GbzError(EINVAL, "unsupported proof shape 2^%d at rate %d" % (logn, rate))
        if out is None:
            out = np.zeros(nbytes, dtype=np.uint8)
        w = _fe(witness)
        mem = _mem(w)
        cap = out.nbytes if isinstance(out, np.ndarray) else out.numel() * out.element_size()
        self.check(lib.gbz_prove(self.h, _ptr(w), logn, rate, prng_seed, _ptr(out), cap, mem))
        return out


def ntt_get_shape(logn):
    sh = np.zeros(3, dtype=np.int32)
    if lib.gbz_ntt_get_shape(logn, _ptr(sh)) != OK:
        raise GbzError(EINVAL, "no two-pass shape for 2^%d" % logn)
    return tuple(int(x) for x in sh)


def ntt_set_shape(logn, k1, log_cols_a, log_rows_b):
    st = lib.gbz_ntt_set_shape(logn, k1, log_cols_a, log_rows_b)
    if st != OK:
        raise GbzError(st, "invalid NTT shape")


def leader_root(root, nparties):
    """Root of create_tree_blake over {root, 0, ..., 0} of nparties."""
    r = np.ascontiguousarray(root, dtype=np.uint8).reshape(32)
    out = np.zeros(32, dtype=np.uint8)
    lib.gbz_leader_root(_ptr(r), nparties, _ptr(out))
    return out


def prove_launches(logn, rate):
    return int(lib.gbz_prove_launches(logn, rate))


def split_levels(flat, N):
    levels, off, cnt = [], 0, N // 4
    while cnt >= 1:
        levels.append(flat[off:off + cnt])
        off += cnt
        cnt //= 2
    return levels


def open_tree_blake(flat_levels, N, pos):
    flat_levels = np.ascontiguousarray(flat_levels, dtype=np.uint8)
    depth = (N // 4).bit_length() - 1
    path = np.zeros((max(depth, 1), 32), dtype=np.uint8)
    d = ctypes.c_uint32()
    st = lib.gbz_merkle_open_blake(_ptr(flat_levels), N, pos, _ptr(path), ctypes.byref(d))
    if st != OK:
        raise GbzError(st, "open_tree_blake: position out of range")
    return path[: d.value]


def transcript_bytes(logn, rate):
    return int(lib.gbz_prove_transcript_bytes(logn, rate))


def hash_to_field(state, elems):
    """hash_to_field with an explicit chain state (numpy uint64[2], updated)."""
    elems = np.ascontiguousarray(elems, dtype=np.uint64).reshape(-1, 2)
    out = np.zeros(2, dtype=np.uint64)
    lib.gbz_hash_to_field(_ptr(state), _ptr(elems), elems.shape[0], _ptr(out))
    return out


class Prng(ctypes.Structure):
    """The glibc random() stream that F::_random and rand() draw from."""
    _fields_ = [("tbl", ctypes.c_int32 * 31), ("f", ctypes.c_int32), ("r", ctypes.c_int32)]

    def __init__(self, seed=1):
        super().__init__()
        lib.gbz_prng_seed(ctypes.addressof(self), seed)

    def next(self):
        return lib.gbz_prng_next(ctypes.addressof(self))

    def field(self):
        out = np.zeros(2, dtype=np.uint64)
        lib.gbz_prng_field(ctypes.addressof(self), _ptr(out))
        return out


def whir_batch_schedule(sizes, rate, whir_k=4):
    """(kappas, merge flags, codeword length per array, transcript bytes) of
    Whir_Batch_Open for these sizes, or None when the reference cannot run
    them (gbz_whir_batch_schedule)."""
    k = len(sizes)
    sz = np.ascontiguousarray(sizes, dtype=np.uint64)
    steps = ctypes.c_int(0)
    kap, agg = np.zeros(64, dtype=np.int32), np.zeros(64, dtype=np.int32)
    cwl, nb = np.zeros(max(k, 1), dtype=np.uint64), ctypes.c_uint64(0)
    rc = lib.gbz_whir_batch_schedule(k, _ptr(sz), rate, whir_k, ctypes.byref(steps), _ptr(kap), _ptr(agg),
                                     _ptr(cwl), ctypes.byref(nb))
    if rc != OK:
        return None
    n = steps.value
    return [int(x) for x in kap[:n]], [int(x) for x in agg[:n]], [int(x) for x in cwl[:k]], int(nb.value)


def field_ops_host(a, b):
    a, b = _fe(a), _fe(b)
    n = a.shape[0]
    outs = [fe_array(n) for _ in range(3)]
    lib.gbz_field_ops_host(_ptr(a), _ptr(b), n, *[_ptr(o) for o in outs])
    return outs


def _rates(rates):
    r0 = np.array([r[0] for r in rates], dtype=np.int32)
    r1 = np.array([r[1] if len(r) > 1 else 0 for r in rates], dtype=np.int32)
    return r0, r1


def pcs_schedule(N, M, rates):
    """prepare_parameters (coPCS.cpp:38-72): (degrees, queries, random shares per party)."""
    r0, r1 = _rates(rates)
    k = len(rates)
    deg, q, rnd = np.zeros(k, dtype=np.int32), np.zeros(k, dtype=np.int32), ctypes.c_uint64(0)
    st = lib.gbz_pcs_schedule(N, M, k, _ptr(r0), _ptr(r1), _ptr(deg), _ptr(q), ctypes.byref(rnd))
    if st != OK:
        raise GbzError(st, "gbz_pcs_schedule rejected N=%d M=%d" % (N, M))
    return [int(x) for x in deg], [int(x) for x in q], int(rnd.value)


class WhirSlot(ctypes.Structure):
    """gbz_whir_slot: one WHIR batch slot the PIOP-mode opening fills."""
    _fields_ = [("arr", ctypes.c_void_p), ("codeword", ctypes.c_void_p), ("betas", ctypes.c_void_p),
                ("claim", ctypes.c_void_p), ("root", ctypes.c_void_p)]


class PcsCommitment:
    """A collaborative-PCS commitment of N parties held on the device (gbz_pcs)."""

    def __init__(self, ctx, h, N, M, rates):
        self.ctx, self.h, self.N, self.M, self.rates = ctx, h, N, M, rates
        b, rl, cl, tb = ctypes.c_int(0), ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        ctx.check(lib.gbz_pcs_info(h, ctypes.byref(b), ctypes.byref(rl), ctypes.byref(cl), ctypes.byref(tb)))
        self.batches, self.row_len, self.codeword_len = b.value, rl.value, cl.value
        self.open_bytes = tb.value

    def data(self, party):
        """(Commit_data rows, codewords, column-root tree levels) of one party."""
        rows = np.zeros((self.batches, self.row_len, 2), dtype=np.uint64)
        cws = np.zeros((self.batches, self.codeword_len, 2), dtype=np.uint64)
        lv = np.zeros((2 * self.codeword_len - 1, 32), dtype=np.uint8)
        self.ctx.check(lib.gbz_pcs_commit_data(self.ctx.h, self.h, party, _ptr(rows), _ptr(cws), _ptr(lv), MEM_HOST))
        return rows, cws, lv

    def claim(self, r):
        """F_ip of the committed data at r (MPI_utils.cpp:483-553): K."""
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
        K = np.zeros(2, dtype=np.uint64)
        self.ctx.check(lib.gbz_pcs_claim(self.ctx.h, self.h, _ptr(r), r.shape[0], _ptr(K), MEM_HOST))
        return K

    def open(self, r, K, fs):
        """PCS_open_new's parties + aggregation: (transcript bytes, fs after)."""
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
        K = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
        f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
        tr = np.zeros(self.open_bytes, dtype=np.uint8)
        self.ctx.check(lib.gbz_pcs_open(self.ctx.h, self.h, _ptr(r), r.shape[0], _ptr(K), _ptr(f), _ptr(tr),
                                        self.open_bytes, MEM_HOST))
        return tr.tobytes(), f

    def open_full(self, r, K, fs, prng):
        """The whole of PCS_open_new, the leader's tail included: (transcript
        bytes, fs after, flags).  prng (a Prng: the leader's random() stream
        when the opening starts) is advanced in place."""
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
        K = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
        f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
        nb = ctypes.c_uint64(0)
        self.ctx.check(lib.gbz_pcs_open_full_bytes(self.h, ctypes.byref(nb)))
        tr = np.zeros(nb.value, dtype=np.uint8)
        flags = ctypes.c_uint32(0)
        st = lib.gbz_pcs_open_full(self.ctx.h, self.h, _ptr(r), r.shape[0], _ptr(K), _ptr(f),
                                   ctypes.addressof(prng), ctypes.byref(flags), _ptr(tr), nb.value, MEM_HOST)
        self.ctx.check(st)
        return tr.tobytes(), f, flags.value

    def claim_piop(self, b1, b2, b3):
        """F_ip of the committed data with input vectors (b2's last
        _queries[0] entries as zero): K."""
        vec = lambda a: np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2)
        b1, b2, b3 = vec(b1), vec(b2), vec(b3)
        K = np.zeros(2, dtype=np.uint64)
        self.ctx.check(lib.gbz_pcs_claim_piop(self.ctx.h, self.h, _ptr(b1), b1.shape[0], _ptr(b2), b2.shape[0],
                                              _ptr(b3), b3.shape[0], _ptr(K), MEM_HOST))
        return K

    def open_piop(self, b1, b2, b3, lagrange, K, fs, prng, slots=True):
        """PCS_open_new in the PIOP mode (isPIOP = true, as coPIOP_prove calls
        it) with input vectors b1, b2, b3 and b2's Lagrange factors (a list of
        arrays): (transcript bytes, fs after, flags, slots) where slots is a
        list of two dicts (arr, codeword, betas, claim, root) or None.  prng
        is advanced in place."""
        vec = lambda a: np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2)
        b1, b2, b3 = vec(b1), vec(b2), vec(b3)
        lag = [vec(x) for x in lagrange]
        logs = (ctypes.c_int * len(lag))(*[int(x.shape[0]).bit_length() - 1 for x in lag])
        cat = np.ascontiguousarray(np.concatenate(lag), dtype=np.uint64)
        K = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
        f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
        nb, sl = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self.ctx.check(lib.gbz_pcs_open_piop_bytes(self.h, logs, len(lag), ctypes.byref(nb), ctypes.byref(sl)))
        tr = np.zeros(nb.value, dtype=np.uint8)
        flags = ctypes.c_uint32(0)
        out, cs = None, None
        if slots:
            md = sl.value
            out = [{"arr": np.zeros((md, 2), np.uint64), "codeword": np.zeros((4 * md, 2), np.uint64),
                    "betas": np.zeros((md, 2), np.uint64), "claim": np.zeros(2, np.uint64),
                    "root": np.zeros(32, np.uint8)} for _ in range(2)]
            cs = (WhirSlot * 2)()
            for c in range(2):
                for k in ("arr", "codeword", "betas", "claim"):
                    setattr(cs[c], k, out[c][k].ctypes.data)
                cs[c].root = out[c]["root"].ctypes.data
        st = lib.gbz_pcs_open_piop(self.ctx.h, self.h, _ptr(b1), b1.shape[0], _ptr(b2), b2.shape[0], _ptr(b3),
                                   b3.shape[0], _ptr(cat), logs, len(lag), _ptr(K), _ptr(f), ctypes.addressof(prng),
                                   ctypes.byref(flags), cs, _ptr(tr), nb.value, MEM_HOST)
        self.ctx.check(st)
        return tr.tobytes(), f, flags.value, out

    def free(self):
        if self.h:
            lib.gbz_pcs_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def pcs_commit(ctx, N, M, rates, shares, random):
    """PCS_commit (coPCS.cpp:236-250) of N parties: (commitment, party roots, leader root)."""
    r0, r1 = _rates(rates)
    sh = np.ascontiguousarray(shares, dtype=np.uint64)
    rn = np.ascontiguousarray(random, dtype=np.uint64)
    h = ctypes.c_void_p()
    roots = np.zeros((N, 32), dtype=np.uint8)
    leader = np.zeros(32, dtype=np.uint8)
    ctx.check(lib.gbz_pcs_commit(ctx.h, N, M, len(rates), _ptr(r0), _ptr(r1), _ptr(sh), _ptr(rn), MEM_HOST,
                                 ctypes.byref(h), _ptr(roots), _ptr(leader)))
    return PcsCommitment(ctx, h, N, M, rates), roots, leader


def cosumcheck(ctx, form, N, p1, p2, R, K, K_r, degrees, p3=None, r1=None, r2=None, fs=(0, 0)):
    """quadratic_coSumcheck / cubic_coSumcheck (coSumcheck.cpp:233, :335) of N
    parties (party-major arrays): (claims [(eval, r)], flags, transcript, fs)."""
    a = [np.ascontiguousarray(x, dtype=np.uint64) for x in (p1, p2)]
    n = a[0].size // (2 * N)
    deg = np.ascontiguousarray(degrees, dtype=np.int32)
    rows = 4 if form == SC_CUBIC else 5
    Rr = np.ascontiguousarray(R, dtype=np.uint64)
    P3 = None if p3 is None else np.ascontiguousarray(p3, dtype=np.uint64)
    R1 = None if r1 is None else np.ascontiguousarray(r1, dtype=np.uint64).reshape(-1, 2)
    R2 = None if r2 is None else np.ascontiguousarray(r2, dtype=np.uint64).reshape(-1, 2)
    Kk = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
    Kr = np.ascontiguousarray(K_r, dtype=np.uint64).reshape(2)
    f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
    cl = np.zeros((rows, len(degrees) + 2, 2), dtype=np.uint64)
    flags = ctypes.c_uint32(0)
    nb = lib.gbz_cosumcheck_transcript_bytes(form, N, _ptr(deg), len(degrees))
    tr = np.zeros(nb, dtype=np.uint8)
    ctx.check(lib.gbz_cosumcheck(ctx.h, form, N, n, _ptr(a[0]), _ptr(a[1]), _ptr(P3), _ptr(Rr), _ptr(R1),
                                 0 if R1 is None else R1.shape[0], _ptr(R2), _ptr(Kk), _ptr(Kr), _ptr(deg),
                                 len(degrees), _ptr(f), _ptr(cl), ctypes.byref(flags), _ptr(tr), nb, MEM_HOST))
    claims = [(cl[i, 0], cl[i, 1:]) for i in range(rows)]
    return claims, flags.value, tr.tobytes(), f


class R1cs:
    """The parties' R1CS rows on the device (gbz_r1cs_create): per matrix A,
    B, C a CSR (row pointers over N x rows rows, columns)."""

    def __init__(self, ctx, N, rows, logm, ptrs, cols):
        self.ctx, self.N, self.rows, self.logm = ctx, N, rows, logm
        self._p = [np.ascontiguousarray(p, dtype=np.uint32) for p in ptrs]
        self._c = [np.ascontiguousarray(c, dtype=np.uint32) for c in cols]
        P = (ctypes.c_void_p * 3)(*[x.ctypes.data for x in self._p])
        C = (ctypes.c_void_p * 3)(*[x.ctypes.data if x.size else None for x in self._c])
        nnz = np.array([x.size for x in self._c], dtype=np.uint64)
        self.h = ctypes.c_void_p()
        ctx.check(lib.gbz_r1cs_create(ctx.h, N, rows, logm, P, C, _ptr(nnz), ctypes.byref(self.h)))

    def reduce(self, r, degrees1):
        """_reduce_R1CS_matrixes_multivariate at r (one entry per degree):
        (RA, RB, RC), each N x rows."""
        r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
        deg = np.ascontiguousarray(degrees1, dtype=np.int32)
        outs = [np.zeros((self.N, self.rows, 2), dtype=np.uint64) for _ in range(3)]
        self.ctx.check(lib.gbz_r1cs_reduce(self.ctx.h, self.h, _ptr(r), r.shape[0], _ptr(deg), len(deg),
                                           *[_ptr(o) for o in outs], MEM_HOST))
        return outs

    def free(self):
        if self.h:
            lib.gbz_r1cs_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def piop_phase1(ctx, N, vL, vR, vO, masks, R1, degrees, fs, vectors=False):
    """prove_phase1 (coPIOP.cpp:241-346) of N parties: (claims [(eval,
    point)], ip N x sum 4d, ip_b1, flags, transcript, fs[, vectors])."""
    a = [np.ascontiguousarray(x, dtype=np.uint64) for x in (vL, vR, vO)]
    n = a[0].size // (2 * N)
    m = np.ascontiguousarray(masks, dtype=np.uint64)
    R = np.ascontiguousarray(R1, dtype=np.uint64)
    deg = np.ascontiguousarray(degrees, dtype=np.int32)
    f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
    cl = np.zeros((4, len(deg) + 2, 2), dtype=np.uint64)
    ip = np.zeros((N, 4 * int(deg.sum()), 2), dtype=np.uint64)
    b1 = np.zeros((N // 4, 2), dtype=np.uint64)
    vec = np.zeros((3, N, 2 * n, 2), dtype=np.uint64) if vectors else None
    flags = ctypes.c_uint32(0)
    nb = lib.gbz_piop_phase1_bytes(N, n, _ptr(deg), len(deg))
    tr = np.zeros(nb, dtype=np.uint8)
    ctx.check(lib.gbz_piop_phase1(ctx.h, N, n, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(m), _ptr(R), _ptr(deg),
                                  len(deg), _ptr(f), _ptr(cl), _ptr(ip), _ptr(b1), _ptr(vec), ctypes.byref(flags),
                                  _ptr(tr), nb, MEM_HOST))
    claims = [(cl[i, 0], cl[i, 1:]) for i in range(4)]
    out = (claims, ip, b1, flags.value, tr.tobytes(), f)
    return out + (vec,) if vectors else out


def piop_phase2(ctx, N, w, masks, r1cs, mask_l, R2, point1, evals1, degrees1, degrees2, K, fs, vectors=False):
    """prove_phase2 (coPIOP.cpp:406-627) of N parties: (claims [(eval,
    point)], abc, ip2, ip3, ip_b1, flags, transcript, fs[, vectors])."""
    w = np.ascontiguousarray(w, dtype=np.uint64)
    nw = w.size // (2 * N)
    m = np.ascontiguousarray(masks, dtype=np.uint64)
    R = np.ascontiguousarray(R2, dtype=np.uint64)
    pt = np.ascontiguousarray(point1, dtype=np.uint64).reshape(-1, 2)
    ev = np.ascontiguousarray(evals1, dtype=np.uint64).reshape(-1, 2)
    d1 = np.ascontiguousarray(degrees1, dtype=np.int32)
    d2 = np.ascontiguousarray(degrees2, dtype=np.int32)
    Kk = np.ascontiguousarray(K, dtype=np.uint64).reshape(2)
    f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
    cl = np.zeros((5, len(d2) + 2, 2), dtype=np.uint64)
    abc = np.zeros((3, 2), dtype=np.uint64)
    ip2 = np.zeros((N, 2 * int(d2.sum()), 2), dtype=np.uint64)
    ip3 = np.zeros((N, 12, 2), dtype=np.uint64)
    b1 = np.zeros((N // 4, 2), dtype=np.uint64)
    vec = np.zeros((2, N, 2 * nw, 2), dtype=np.uint64) if vectors else None
    flags = ctypes.c_uint32(0)
    nb = lib.gbz_piop_phase2_bytes(N, _ptr(d2), len(d2))
    tr = np.zeros(nb, dtype=np.uint8)
    ctx.check(lib.gbz_piop_phase2(ctx.h, N, nw, _ptr(w), _ptr(m), r1cs.h, mask_l, _ptr(R), _ptr(pt), _ptr(ev),
                                  _ptr(d1), len(d1), _ptr(d2), len(d2), _ptr(Kk), _ptr(f), _ptr(cl), _ptr(abc),
                                  _ptr(ip2), _ptr(ip3), _ptr(b1), _ptr(vec), ctypes.byref(flags), _ptr(tr), nb,
                                  MEM_HOST))
    claims = [(cl[i, 0], cl[i, 1:]) for i in range(5)]
    out = (claims, abc, ip2, ip3, b1, flags.value, tr.tobytes(), f)
    return out + (vec,) if vectors else out


VERIFY_CHECKS = ("layout", "point", "sumcheck_sum", "sumcheck_challenge", "sumcheck_final", "whir_sum",
                 "whir_challenge", "queries", "answers", "combine", "whir_K", "final_point", "step2", "step3")


def verify_proof(transcript, logn, rate, prng_seed=1):
    """gbz_verify_proof: (ok, names of the failed checks)."""
    tr = np.frombuffer(bytes(transcript), dtype=np.uint8)
    failed = ctypes.c_uint32(0)
    st = lib.gbz_verify_proof(_ptr(tr), tr.size, logn, rate, prng_seed, ctypes.byref(failed))
    if st not in (0, 4):
        raise GbzError(st, "gbz_verify_proof: bad arguments")
    return st == 0, [n for i, n in enumerate(VERIFY_CHECKS) if failed.value >> i & 1]


def dpcs_batch_commit(ctx, arr, arr2, rate, batch):
    """Batch_dCommit (distributed_PCS.cpp:56-147) of N parties (arr, arr2:
    N x A): (commit_data, codewords N x batch x L, levels N x (2L-1) x 32,
    roots N x 32, leader root)."""
    arr = np.ascontiguousarray(arr, dtype=np.uint64)
    arr2 = np.ascontiguousarray(arr2, dtype=np.uint64)
    N, A = arr.shape[0], arr.shape[1]
    L = A // batch * rate
    cd = np.zeros_like(arr2)
    cw = np.zeros((N, batch, L, 2), dtype=np.uint64)
    lv = np.zeros((N, 2 * L - 1, 32), dtype=np.uint8)
    roots = np.zeros((N, 32), dtype=np.uint8)
    lead = np.zeros(32, dtype=np.uint8)
    ctx.check(lib.gbz_dpcs_batch_commit(ctx.h, N, A, _ptr(arr), _ptr(arr2), rate, batch, _ptr(cd), _ptr(cw), _ptr(lv),
                                        _ptr(roots), _ptr(lead), MEM_HOST))
    return cd, cw, lv, roots, lead


def dpcs_open(ctx, commit_data, codewords, points, claims, rate, whir_rate, fs=(0, 0), verify=True):
    """PIOP_dOpen_batch_new (distributed_PCS.cpp:1175-1534) of N parties:
    commit_data P x N x rows x S, codewords P x N x rows x L.  Returns
    (arr, betas, K, whir codeword, whir root, flags, transcript, fs)."""
    cd = np.ascontiguousarray(commit_data, dtype=np.uint64)
    cw = np.ascontiguousarray(codewords, dtype=np.uint64)
    P, N, rows, S = cd.shape[0], cd.shape[1], cd.shape[2], cd.shape[3]
    pts = np.ascontiguousarray(points, dtype=np.uint64)
    ys = np.ascontiguousarray(claims, dtype=np.uint64)
    lN = N.bit_length() - 1
    D = (1 << (lN - lN // 2)) * (1 << (lN // 2))
    na = N * S // D
    arr = np.zeros((na, 2), dtype=np.uint64)
    bet = np.zeros((na, 2), dtype=np.uint64)
    K = np.zeros(2, dtype=np.uint64)
    wc = np.zeros((na * whir_rate, 2), dtype=np.uint64)
    root = np.zeros(32, dtype=np.uint8)
    f = np.array(np.asarray(fs, dtype=np.uint64).reshape(2), copy=True)
    flags = ctypes.c_uint32(0)
    nb = lib.gbz_dpcs_open_bytes(N, P, rate)
    tr = np.zeros(nb, dtype=np.uint8)
    ctx.check(lib.gbz_dpcs_open(ctx.h, N, P, rows, S, rate, _ptr(cd), _ptr(cw), _ptr(pts), _ptr(ys), int(verify),
                                whir_rate, _ptr(f), _ptr(arr), _ptr(bet), _ptr(K), _ptr(wc), _ptr(root),
                                ctypes.byref(flags), _ptr(tr), nb, MEM_HOST))
    return arr, bet, K, wc, root, flags.value, tr.tobytes(), f


def dpcs_commit(ctx, arr, rate):
    """dCommit (distributed_PCS.cpp:150-170) of N parties (arr: N x A):
    (codeword N x rate A, levels, roots N x 32, leader root)."""
    arr = np.ascontiguousarray(arr, dtype=np.uint64)
    N, A = arr.shape[0], arr.shape[1]
    lN = N.bit_length() - 1
    d = 1 << (lN - lN // 2)
    L = A * rate
    cw = np.zeros((N, L, 2), dtype=np.uint64)
    lv = np.zeros((N, 2 * (L // d) - 1, 32), dtype=np.uint8)
    roots = np.zeros((N, 32), dtype=np.uint8)
    lead = np.zeros(32, dtype=np.uint8)
    ctx.check(lib.gbz_dpcs_commit(ctx.h, N, A, _ptr(arr), rate, _ptr(cw), _ptr(lv), _ptr(roots), _ptr(lead),
                                  MEM_HOST))
    return cw, lv, roots, lead


PCS_UNITS = {32: 32, 33: 32, 37: 4, 46: 32, 47: 4, 63: 32, 64: 4, 68: 32}
# records of the batch opening with units other than a field element
BATCH_UNITS = {19: 4, 22: 4, 23: 32, 24: 32}


def parse_transcript(buf):
    """[(tag, count, payload bytes)] of a transcript."""
    buf = bytes(buf)
    out, off = [], 0
    units = {1: 32, 9: 32, 13: 32, 10: 4, **BATCH_UNITS, **PCS_UNITS}
    while off < len(buf):
        tag, count = np.frombuffer(buf, dtype=np.uint32, count=2, offset=off)
        unit = units.get(int(tag), 16)
        out.append((int(tag), int(count), buf[off + 8: off + 8 + unit * int(count)]))
        off += 8 + unit * int(count)
    return out
