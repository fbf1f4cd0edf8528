"""cusat_gb300 -- GB300-native receive-side FEC path for DVB-S2/S2X.

Soft demapping with deinterleave, layered offset min-sum LDPC decoding on
int16 LLRs with a syndrome early exit, and the BCH syndrome check, as
hand-written sm_103a CUDA kernels behind the C ABI of include/cusat_fec.h.
This module is the Python host side of that ABI.  Its classes keep the names,
arguments and result conventions of the reference's C++ classes for the path:

  ldpc_decode_cuda  lib/cusat_dsp/cuda/ldpc_decode_kernel.cuh:22-107
  ldpc_decode       lib/cusat_dsp/ldpc_decode.h:22-69
  demapper_cuda     lib/cusat_dsp/cuda/demapper_kernel.cuh:23-89
  bch_check_cuda    lib/cusat_dsp/cuda/bch_check_kernel.cuh:9-24

  rx_fec_chain      lib/cusat_dsp/rx_fec_chain.h:61-297
  rx_fec_pool       lib/cusat_dsp/rx_fec_pool.h:25-140
  gpu_decode_budget lib/cusat_dsp/rx_fec_chain.h:52-59

plus ``rx_fec`` (one MODCOD's demap -> decode -> BCH chain).

Device buffers are torch CUDA tensors (or raw device addresses as int);
host buffers are numpy arrays.  Streams are torch.cuda.Stream objects, raw
cudaStream_t values as int, or None (legacy default stream).  There is no
CPU fallback: without the built library or a GPU every call raises.
"""
import ctypes

import numpy as np

from . import _capi
from ._capi import CusatError
from .enums import *  # noqa: F401,F403
from .enums import FECFRAME_NORMAL, FECFRAME_SHORT, FECFRAME_MEDIUM  # noqa: F401

__all__ = ["ldpc_decode_cuda", "ldpc_decode", "demapper_cuda", "bch_check_cuda", "rx_fec", "batch", "server",
           "generator", "bb_extractor", "pl_extractor", "pl_layout", "pl_rotation_index", "gpu_decode_budget", "rx_fec_chain", "rx_fec_pool", "dd_snr",
           "code_info", "modcod_info", "encode_frames", "map_frames", "capped_llr_gain",
           "CusatError", "library_path"]


def library_path():
    return _capi.LIB_PATH


def _addr(x):
    """Device/host address of a torch tensor, numpy array, int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    if hasattr(s, "cuda_stream"):
        return s.cuda_stream
    raise TypeError(f"not a stream: {type(s)}")


def _host(a, dtype, n):
    a = np.ascontiguousarray(a, dtype)
    if a.size < n:
        raise ValueError(f"host buffer holds {a.size} elements, {n} needed")
    return a


def _info(fn, handle, n):
    out = np.zeros(n, np.int32)
    _capi.check(fn(handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
    return [int(v) for v in out]


def code_info(framesize, rate):
    """Dimensions of the (framesize, rate) code: n_ldpc, k_ldpc, k_bch, n_bch,
    t, bch_degree, q, n_steps, lanes, cmax, edges, cnt_max."""
    L = _capi.lib()
    out = np.zeros(12, np.int32)
    _capi.check(L.cusat_code_info(framesize, rate, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
    keys = ["n_ldpc", "k_ldpc", "k_bch", "n_bch", "t", "bch_degree", "q", "n_steps", "lanes", "cmax",
            "edges", "cnt_max"]
    return dict(zip(keys, (int(v) for v in out)))


def modcod_info(modulation, rate, framesize):
    """Constellation points (complex64, by label), interleaver column offsets
    and frame geometry of a MODCOD."""
    L = _capi.lib()
    pts = np.zeros(2 * 256, np.float32)
    col = np.zeros(8, np.uint32)
    out = np.zeros(6, np.int32)
    _capi.check(L.cusat_modcod_info(modulation, rate, framesize, pts.ctypes.data, col.ctypes.data,
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
    n_mod, n_points, fec_len, xfec, il, kind = (int(v) for v in out)
    p = pts[:2 * n_points]
    return {"n_mod": n_mod, "n_points": n_points, "fecframe_len": fec_len, "xfecframe_len": xfec,
            "interleaved_len": il, "kind": kind, "points": (p[0::2] + 1j * p[1::2]).astype(np.complex64),
            "col_offset": col}


def capped_llr_gain(modulation, rate, framesize, llr_gain):
    return float(_capi.lib().cusat_modcod_capped_llr_gain(modulation, rate, framesize, llr_gain))


def encode_frames(framesize, rate, msg):
    """BCH + LDPC encode k_bch/8-byte messages into n_ldpc/8-byte codewords."""
    ci = code_info(framesize, rate)
    msg = np.ascontiguousarray(msg, np.uint8).reshape(-1, ci["k_bch"] // 8)
    cw = np.zeros((msg.shape[0], ci["n_ldpc"] // 8), np.uint8)
    _capi.check(_capi.lib().cusat_gen_encode(framesize, rate, msg.ctypes.data, cw.ctypes.data, msg.shape[0]))
    return cw


def map_frames(modulation, rate, framesize, cw):
    """Interleave + map codewords to symbols: float32 [B, xfecframe_len * 2]."""
    mi = modcod_info(modulation, rate, framesize)
    cw = np.ascontiguousarray(cw, np.uint8).reshape(-1, mi["fecframe_len"] // 8)
    sym = np.zeros((cw.shape[0], mi["xfecframe_len"] * 2), np.float32)
    _capi.check(_capi.lib().cusat_gen_map(modulation, rate, framesize, cw.ctypes.data, cw.shape[0],
                                          sym.ctypes.data))
    return sym



def _weights_arg(weights):
    """(pointer, n_iter, keep-alive array) for a learned weight table
    ([n_iter, 32, 2] int16 {beta, alpha/64}) or None (plain decoder)."""
    if weights is None:
        return None, 0, None
    w = np.ascontiguousarray(np.asarray(weights, np.int16).reshape(-1, 32, 2))
    return w.ctypes.data, w.shape[0], w

class ldpc_decode_cuda:
    """Layered min-sum LDPC decoder (reference cuda::ldpc_decode_cuda).

    ``decode_launch_async`` is the asynchronous device path; ``decode_batch``
    and ``decode_batch_d2h`` are the synchronous host-result paths.  Trials
    are max_trials - iterations used, or -1 when not converged."""

    def __init__(self, framesize, rate, max_trials=25, max_batch=64):
        L = _capi.lib()
        h = ctypes.c_void_p()
        _capi.check(L.cusat_ldpc_decoder_create(framesize, rate, max_trials, max_batch, ctypes.byref(h)))
        self._h = h
        info = _info(L.cusat_ldpc_decoder_info, h, 8)
        self.framesize, self.rate = framesize, rate
        self._n, self._k, self._kb, self.q, self.n_steps, self.max_trials, self.max_batch, self.lanes = info

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_ldpc_decoder_destroy(self._h)
            self._h = None

    __del__ = close

    def n_bits(self):
        return self._n

    def k_bits(self):
        return self._k

    def k_bytes(self):
        return self._kb

    def decode_launch_async(self, soft_in, batch_size, stream=None, hard_out=None, result_out=None):
        _capi.check(_capi.lib().cusat_ldpc_decode_launch(self._h, _addr(soft_in), batch_size, _stream(stream),
                                                          _addr(hard_out), _addr(result_out)))

    def set_weights(self, weights):
        """Learned min-sum weights ([n_iter, 32, 2] int16 {beta, alpha/64}) or None."""
        p, n, _keep = _weights_arg(weights)
        _capi.check(_capi.lib().cusat_ldpc_decoder_set_weights(self._h, p, n))

    def set_max_ctas(self, max_ctas):
        """Caps the persistent grid (0 = no cap): each CTA then decodes
        several frames of a batch in turn."""
        _capi.check(_capi.lib().cusat_ldpc_decoder_set_max_ctas(self._h, max_ctas))

    def set_frames_per_cta(self, n):
        """0: by batch size (frame pairs once every SM receives one), 1: one
        frame per CTA, 2: frame pairs whenever the code allows them."""
        _capi.check(_capi.lib().cusat_ldpc_decoder_set_frames_per_cta(self._h, n))

    def frames_per_cta(self, batch_size):
        """Frames per CTA a launch of batch_size frames runs: 2 for frame
        pairs (short frames, no learned weights), else 1."""
        n = _capi.lib().cusat_ldpc_decoder_frames_per_cta(self._h, batch_size)
        _capi.check(min(n, 0))
        return n

    def results(self, batch_size):
        hard = np.zeros((batch_size, self._kb), np.uint8)
        trials = np.zeros(batch_size, np.int32)
        _capi.check(_capi.lib().cusat_ldpc_decoder_results(self._h, hard.ctypes.data, trials.ctypes.data,
                                                           batch_size))
        return hard, trials

    def decode_batch(self, soft_in, batch_size=None, stream=None):
        soft = np.ascontiguousarray(soft_in, np.int16).reshape(-1, self._n)
        b = soft.shape[0] if batch_size is None else batch_size
        hard = np.zeros((b, self._kb), np.uint8)
        trials = np.zeros(b, np.int32)
        _capi.check(_capi.lib().cusat_ldpc_decode_batch(self._h, soft.ctypes.data, hard.ctypes.data,
                                                        trials.ctypes.data, b, _stream(stream)))
        return hard, trials

    def decode_batch_d2h(self, soft_in_dev, batch_size, stream=None):
        hard = np.zeros((batch_size, self._kb), np.uint8)
        trials = np.zeros(batch_size, np.int32)
        _capi.check(_capi.lib().cusat_ldpc_decode_batch_d2h(self._h, _addr(soft_in_dev), hard.ctypes.data,
                                                            trials.ctypes.data, batch_size, _stream(stream)))
        return hard, trials


class ldpc_decode(ldpc_decode_cuda):
    """Standalone decoder (reference cusat_dsp::ldpc_decode): owns a stream."""

    def __init__(self, framesize, rate, max_trials=25, cuda_max_batch=64):
        super().__init__(framesize, rate, max_trials, cuda_max_batch)
        import torch
        self._stream = torch.cuda.Stream()

    def cuda_stream(self):
        return self._stream

    def n_bytes(self):
        return self._n // 8

    def decode_batch_cuda(self, soft_in, batch_size=None):
        return self.decode_batch(soft_in, batch_size, self._stream)

    def decode_batch_cuda_d2h(self, soft_in_dev, batch_size):
        return self.decode_batch_d2h(soft_in_dev, batch_size, self._stream)


class demapper_cuda:
    """Soft demapper + deinterleaver (reference cuda::demapper_cuda)."""

    def __init__(self, constellation, rate, framesize, max_batch=64):
        L = _capi.lib()
        h = ctypes.c_void_p()
        _capi.check(L.cusat_demapper_create(constellation, rate, framesize, max_batch, ctypes.byref(h)))
        self._h = h
        self._fec, self._xfec, self._nmod, self._il = _info(L.cusat_demapper_info, h, 4)
        self.max_batch = max_batch

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_demapper_destroy(self._h)
            self._h = None

    __del__ = close

    def fecframe_len(self):
        return self._fec

    def xfecframe_len(self):
        return self._xfec

    def n_mod(self):
        return self._nmod

    def capped_llr_gain(self, llr_gain):
        return float(_capi.lib().cusat_demapper_capped_llr_gain(self._h, llr_gain))

    def soft_out_dev(self):
        """Device address of the internal LLR buffer."""
        return int(_capi.lib().cusat_demapper_soft_out_dev(self._h))

    def demap_launch(self, sym_dev, batch_size, noise_var, llr_gain, soft_out_dev=None, stream=None):
        _capi.check(_capi.lib().cusat_demap_launch(self._h, _addr(sym_dev), batch_size, noise_var, llr_gain,
                                                   _addr(soft_out_dev), _stream(stream)))

    def demap_batch_async(self, sym_in_host, batch_size, noise_var, llr_gain, stream=None):
        sym = _host(sym_in_host, np.float32, batch_size * self._xfec * 2)
        self._keep = sym
        _capi.check(_capi.lib().cusat_demap_batch_async(self._h, sym.ctypes.data, batch_size, noise_var,
                                                        llr_gain, _stream(stream)))

    def demap_batch(self, sym_in_host, batch_size, noise_var, llr_gain):
        sym = _host(sym_in_host, np.float32, batch_size * self._xfec * 2)
        _capi.check(_capi.lib().cusat_demap_batch(self._h, sym.ctypes.data, batch_size, noise_var, llr_gain))


class bch_check_cuda:
    """BCH syndrome check (reference cuda::bch_check_cuda)."""

    def __init__(self, flat_lut, gen_poly, gen_degree, n_bytes):
        lut = np.ascontiguousarray(flat_lut, np.uint64).reshape(256 * 4)
        gen = np.ascontiguousarray(gen_poly, np.uint64).reshape(4)
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_bch_checker_create(lut.ctypes.data, gen.ctypes.data, gen_degree, n_bytes,
                                                         ctypes.byref(h)))
        self._h = h
        self.degree = gen_degree

    @classmethod
    def for_code(cls, framesize, rate):
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_bch_checker_create_for_code(framesize, rate, ctypes.byref(h)))
        self._h = h
        self.degree = code_info(framesize, rate)["bch_degree"]
        return self

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_bch_checker_destroy(self._h)
            self._h = None

    __del__ = close

    def n_bytes(self):
        return int(_capi.lib().cusat_bch_checker_n_bytes(self._h))

    def check_async(self, codewords_dev, valid_out_dev, batch_size, stream=None, rem_out_dev=None):
        _capi.check(_capi.lib().cusat_bch_check_launch(self._h, _addr(codewords_dev), _addr(valid_out_dev),
                                                       _addr(rem_out_dev), batch_size, _stream(stream)))


class rx_fec:
    """One MODCOD's receive chain: demap + deinterleave, LDPC decode,
    then the BCH check (replaces rx_fec_chain::launch_slot_gpu's launch
    sequence, lib/cusat_dsp/rx_fec_chain.cc:361-505)."""

    def __init__(self, constellation, rate, framesize, max_trials=25, max_batch=64):
        L = _capi.lib()
        h = ctypes.c_void_p()
        _capi.check(L.cusat_rx_fec_create(constellation, rate, framesize, max_trials, max_batch,
                                          ctypes.byref(h)))
        self._h = h
        self.xfec, self.n_bits, self.k_bits, self.k_bytes, self.k_bch, self.n_mod = _info(L.cusat_rx_fec_info,
                                                                                          h, 6)
        self.max_trials, self.max_batch = max_trials, max_batch

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_rx_fec_destroy(self._h)
            self._h = None

    __del__ = close

    def capped_llr_gain(self, llr_gain):
        return float(_capi.lib().cusat_rx_fec_capped_llr_gain(self._h, llr_gain))

    def set_frames_per_cta(self, n):
        """As ldpc_decode_cuda.set_frames_per_cta."""
        _capi.check(_capi.lib().cusat_rx_fec_set_frames_per_cta(self._h, n))

    def set_weights(self, weights):
        """Learned min-sum weights ([n_iter, 32, 2] int16 {beta, alpha/64}) or None."""
        p, n, _keep = _weights_arg(weights)
        _capi.check(_capi.lib().cusat_rx_fec_set_weights(self._h, p, n))

    def launch(self, sym_dev, batch_size, noise_var, llr_gain, hard_out, trials_out, bch_valid_out=None,
               stream=None):
        _capi.check(_capi.lib().cusat_rx_fec_launch(self._h, _addr(sym_dev), batch_size, noise_var, llr_gain,
                                                    _addr(hard_out), _addr(trials_out), _addr(bch_valid_out),
                                                    _stream(stream)))


class batch:
    """Mixed-MODCOD batch decoder: frames of any of `modcods` ((modulation,
    rate, frame size) triples) in one launch sequence (demap -> decode
    -> BCH), optionally captured into a CUDA graph.  No counterpart in the
    reference (one chain per MODCOD, lib/cusat_dsp/rx_fec_pool.cc:48-87)."""

    def __init__(self, modcods, max_trials=50, max_frames=1024):
        arr = np.ascontiguousarray(np.asarray(modcods, np.int32).reshape(-1, 3))
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_batch_create(arr.ctypes.data, arr.shape[0], max_trials, max_frames,
                                                   ctypes.byref(h)))
        self._h = h
        self.modcods = [tuple(int(v) for v in r) for r in arr]
        self.max_trials, self.max_frames = max_trials, max_frames
        self._frames = None

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def info(self):
        return _info(_capi.lib().cusat_batch_info, self._h, 4)

    def set_weights(self, modcod, weights):
        """Learned weights for MODCOD index `modcod` of this batch, or None."""
        p, n, _keep = _weights_arg(weights)
        _capi.check(_capi.lib().cusat_batch_set_weights(self._h, modcod, p, n))

    def set_max_ctas(self, max_ctas):
        """Caps every class's persistent grid (0 = no cap)."""
        _capi.check(_capi.lib().cusat_batch_set_max_ctas(self._h, max_ctas))

    @staticmethod
    def frames(modcod, noise_var, llr_gain, sym, hard, trials, bch_valid=None):
        """Array of cusat_frame from per-frame lists (addresses or tensors)."""
        n = len(modcod)
        arr = (_capi.Frame * n)()
        for i in range(n):
            arr[i] = _capi.Frame(int(modcod[i]), float(noise_var[i]), float(llr_gain[i]), 0, _addr(sym[i]),
                                 _addr(hard[i]), _addr(trials[i]),
                                 None if bch_valid is None else _addr(bch_valid[i]))
        return arr

    def launch(self, frames, stream=None):
        self._frames = frames
        _capi.check(_capi.lib().cusat_batch_launch(self._h, ctypes.addressof(frames), len(frames),
                                                   _stream(stream)))

    def tune(self, frames, reps=3, stream=None):
        best = ctypes.c_float()
        _capi.check(_capi.lib().cusat_batch_tune(self._h, ctypes.addressof(frames), len(frames), reps,
                                                 _stream(stream), ctypes.byref(best)))
        return best.value

    def tuned(self):
        """The tuned launch configuration: one dict per kernel class."""
        out = np.zeros(5 * 64, np.int32)
        solo = np.zeros(64, np.float32)
        n = _capi.lib().cusat_batch_tuned(self._h, out.ctypes.data, solo.ctypes.data, 64)
        _capi.check(min(n, 0))
        res = []
        for k in range(n):
            cmax, lanes, frames, grid, pos = (int(v) for v in out[5 * k:5 * k + 5])
            res.append({"slots": cmax, "lanes": lanes, "frames": frames, "ctas": grid,
                        "frames_per_cta": frames / grid if grid else None, "order": pos,
                        "solo_ms": float(solo[k])})
        return res

    def capture(self, frames, stream):
        self._frames = frames
        _capi.check(_capi.lib().cusat_batch_capture(self._h, ctypes.addressof(frames), len(frames),
                                                    _stream(stream)))

    def replay(self, stream):
        _capi.check(_capi.lib().cusat_batch_replay(self._h, _stream(stream)))


# cusat_result as a numpy record (48 bytes, the C layout)
_RESULT = np.dtype([("tag", "<u8"), ("modcod", "<i4"), ("trials", "<i4"), ("bch_valid", "<i4"), ("reserved", "<i4"),
                    ("arrival_s", "<f8"), ("admit_s", "<f8"), ("done_s", "<f8")])


import collections as _collections  # noqa: E402

ServerResult = _collections.namedtuple("ServerResult", list(_RESULT.names))


class server:
    """Serving loop (continuous batching, HBM-budget admission) over the
    mixed-MODCOD decoder; see cusat_server_create in include/cusat_fec.h."""

    HOST_SYMBOLS = 1

    def __init__(self, modcods, max_trials=50, hbm_budget=1 << 30, slots=4, max_batch=512):
        arr = np.ascontiguousarray(np.asarray(modcods, np.int32).reshape(-1, 3))
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_server_create(arr.ctypes.data, arr.shape[0], max_trials, int(hbm_budget),
                                                    slots, max_batch, ctypes.byref(h)))
        self._h = h
        self.modcods = [tuple(int(v) for v in r) for r in arr]

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_server_destroy(self._h)
            self._h = None

    __del__ = close

    def now(self):
        return float(_capi.lib().cusat_server_now(self._h))

    def set_weights(self, modcod, weights):
        p, n, _keep = _weights_arg(weights)
        _capi.check(_capi.lib().cusat_server_set_weights(self._h, modcod, p, n))

    @staticmethod
    def requests(modcod, noise_var, llr_gain, sym, tag, arrival_s=None, hard_host=None, flags=0):
        """Array of cusat_request from per-request lists (addresses or tensors)."""
        n = len(modcod)
        arr = (_capi.Request * n)()
        for i in range(n):
            arr[i] = _capi.Request(int(modcod[i]), float(noise_var[i]), float(llr_gain[i]), flags, _addr(sym[i]),
                                   None if hard_host is None else _addr(hard_host[i]), int(tag[i]),
                                   -1.0 if arrival_s is None else float(arrival_s[i]))
        return arr

    def submit(self, reqs):
        """Queues the requests (copied by the library; the symbols and host
        hard-bit buffers they point to must stay valid until their results)."""
        _capi.check(_capi.lib().cusat_server_submit(self._h, ctypes.addressof(reqs), len(reqs)))

    def poll(self, max_results=4096, wait_ms=10):
        """Completed results (namedtuples with the cusat_result fields)."""
        out = (_capi.Result * max_results)()
        n = _capi.lib().cusat_server_poll(self._h, ctypes.addressof(out), max_results, wait_ms)
        if n < 0:
            _capi.check(n)
        rec = np.frombuffer(out, dtype=_RESULT, count=n)
        return [ServerResult(*r) for r in rec.tolist()]

    def stats(self):
        out = (ctypes.c_double * 8)()
        _capi.check(_capi.lib().cusat_server_stats(self._h, out))
        keys = ["pending", "batches", "frames", "largest_batch", "max_inflight_batches", "peak_bytes",
                "budget_bytes", "inflight_batches"]
        return dict(zip(keys, list(out)))


class generator:
    """Transmitter on the GPU: BCH + LDPC encode and map a batch of messages
    (device memory in and out); equal bit for bit to encode_frames and
    map_frames."""

    def __init__(self, constellation, rate, framesize, max_batch=256):
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_generator_create(constellation, rate, framesize, max_batch, ctypes.byref(h)))
        self._h = h
        self.msg_bytes, self.cw_bytes, self.xfec, self.max_batch = _info(_capi.lib().cusat_generator_info, h, 4)

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_generator_destroy(self._h)
            self._h = None

    __del__ = close

    def generate(self, msg_dev, batch, cw_dev, sym_dev=None, stream=None):
        _capi.check(_capi.lib().cusat_generate(self._h, _addr(msg_dev), batch, _addr(cw_dev), _addr(sym_dev),
                                               _stream(stream)))


class bb_extractor:
    """Post-FEC baseband stage of one code: drop failed frames, descramble,
    check the BBHEADER and pack the GSE data fields (device memory)."""

    def __init__(self, framesize, rate):
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_bb_extractor_create(framesize, rate, ctypes.byref(h)))
        self._h = h
        self.kbch_bytes = code_info(framesize, rate)["k_bch"] // 8

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_bb_extractor_destroy(self._h)
            self._h = None

    __del__ = close

    def extract(self, hard_dev, hard_stride, trials_dev, bch_valid_dev, batch, out_dev, max_out, lengths_dev,
                offsets_dev, stream=None):
        _capi.check(_capi.lib().cusat_bb_extract(self._h, _addr(hard_dev), hard_stride, _addr(trials_dev),
                                                 _addr(bch_valid_dev), batch, _addr(out_dev), max_out,
                                                 _addr(lengths_dev), _addr(offsets_dev), _stream(stream)))


_PL_KEYS = ["slots", "pilots", "pilot_blocks", "data_symbols", "payload_symbols", "modcod", "framesize",
            "bits_per_symbol", "dummy", "deliverable", "reserved"]


def pl_layout(pls_code):
    """PLFRAME layout of an 8-bit PLS code (reference pl_layout_from_code)."""
    out = np.zeros(11, np.int32)
    _capi.check(_capi.lib().cusat_pl_layout(pls_code, out.ctypes.data))
    return dict(zip(_PL_KEYS, (int(v) for v in out)))


def pl_rotation_index(gold, n):
    """Scrambling rotation index R_n(i), i < n (descrambling factor e^{-j R pi/2})."""
    r = np.zeros(n, np.uint8)
    _capi.check(_capi.lib().cusat_pl_rotation_index(gold, r.ctypes.data, n))
    return r


class pl_extractor:
    """PL receiver tail for located PLFRAMEs (reference
    pl_receiver::process_payload's data step): descramble, drop the pilot
    blocks, counter-rotate each slot -> XFECFRAME data symbols (device)."""

    def __init__(self, gold_codes, max_frames=256):
        g = np.ascontiguousarray(np.asarray(gold_codes, np.int32).reshape(-1))
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_pl_extractor_create(g.ctypes.data, g.size, max_frames, ctypes.byref(h)))
        self._h = h
        self.max_frames = max_frames

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_pl_extractor_destroy(self._h)
            self._h = None

    __del__ = close

    @staticmethod
    def frames(payload, data, pls_code, gold, slot_rot=None):
        """Array of cusat_pl_frame from per-frame lists (addresses or tensors)."""
        n = len(payload)
        arr = (_capi.PlFrame * n)()
        for f in range(n):
            arr[f] = _capi.PlFrame(_addr(payload[f]), _addr(data[f]),
                                   None if slot_rot is None or slot_rot[f] is None else _addr(slot_rot[f]),
                                   int(pls_code[f]), int(gold[f]))
        return arr

    def extract(self, frames, stream=None):
        self._frames = frames
        _capi.check(_capi.lib().cusat_pl_extract(self._h, ctypes.addressof(frames), len(frames), _stream(stream)))


def _symbols(symbols):
    """Host symbols as a contiguous float32 (re, im) array and their count."""
    a = np.asarray(symbols)
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a, np.complex64).view(np.float32)
    else:
        a = np.ascontiguousarray(a, np.float32)
    return a, a.size // 2


def dd_snr(constellation, rate, framesize, symbols, stride=1):
    """Decision-directed SNR (linear) of host symbols: qpsk_snr_dd for QPSK,
    constellation_snr_dd on every stride-th symbol otherwise."""
    a, n = _symbols(symbols)
    out = ctypes.c_float()
    _capi.check(_capi.lib().cusat_dd_snr(constellation, rate, framesize, a.ctypes.data, n, stride,
                                         ctypes.byref(out)))
    return out.value


class gpu_decode_budget:
    """Shared cap on frames in flight across chains (0 = unlimited)."""

    def __init__(self, cap=-1):
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_decode_budget_create(cap, ctypes.byref(h)))
        self._h = h

    @classmethod
    def make_default(cls):
        return cls(-1)

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_decode_budget_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def cap(self):
        return _info(_capi.lib().cusat_decode_budget_info, self._h, 2)[0]

    @property
    def in_flight(self):
        return _info(_capi.lib().cusat_decode_budget_info, self._h, 2)[1]


def _check_ready(rc):
    if rc < 0:
        _capi.check(rc)
    return rc > 0


class rx_fec_chain:
    """One MODCOD's frame-at-a-time receive chain: submit XFECFRAMEs, drain
    completed micro-batches in order, read the GSE data fields."""

    def __init__(self, framesize, rate, constellation, max_trials=25, cuda_max_batch=64, n_gpu_streams=8,
                 micro_batch=4, _handle=None):
        self._owned = _handle is None
        if _handle is None:
            h = ctypes.c_void_p()
            _capi.check(_capi.lib().cusat_rx_chain_create(framesize, rate, constellation, max_trials,
                                                          cuda_max_batch, n_gpu_streams, micro_batch,
                                                          ctypes.byref(h)))
            _handle = h
        self._h = _handle
        info = _info(_capi.lib().cusat_rx_chain_info, self._h, 6)
        self.xfecframe_len, self.kbch_bytes, self._batch_size, self._max_out, self.micro_batch, self.n_streams = info
        self._budget = None

    def close(self):
        if getattr(self, "_h", None):
            if self._owned:
                _capi.lib().cusat_rx_chain_destroy(self._h)
            self._h = None

    __del__ = close

    @staticmethod
    def frame_passes_fec_checks(ldpc_trials_remaining, bch_valid):
        return ldpc_trials_remaining >= 0 and bool(bch_valid)

    def submit_xfecframe(self, symbols, n_symbols=None):
        a, n = _symbols(symbols)
        if n_symbols is not None:
            n = min(n, int(n_symbols))
        return _check_ready(_capi.lib().cusat_rx_chain_submit_xfecframe(self._h, a.ctypes.data, n))

    def drain_completed(self):
        return _check_ready(_capi.lib().cusat_rx_chain_drain_completed(self._h))

    def get_gse_output(self, max_bytes=None):
        if max_bytes is None:
            max_bytes = self._max_out
        out = self._out_buffer(max_bytes)
        n = _capi.lib().cusat_rx_chain_get_gse_output(self._h, out.ctypes.data, max_bytes)
        if n < 0:
            _capi.check(n)
        return out[:n].copy()

    def _out_buffer(self, n):
        # one buffer per object, reused: outputs are copied out of it
        buf = getattr(self, "_buf", None)
        if buf is None or buf.size < max(n, 1):
            buf = self._buf = np.empty(max(n, 1), np.uint8)
        return buf

    def gse_dfl_sizes(self):
        n = _capi.lib().cusat_rx_chain_gse_dfl_sizes(self._h, None, 0)
        if n < 0:
            _capi.check(n)
        out = np.zeros(max(n, 1), np.int32)
        _capi.lib().cusat_rx_chain_gse_dfl_sizes(self._h, out.ctypes.data, n)
        return [int(v) for v in out[:n]]

    def launch_partial(self):
        _capi.check(_capi.lib().cusat_rx_chain_launch_partial(self._h))

    def flush(self):
        _capi.check(_capi.lib().cusat_rx_chain_flush(self._h))

    def reset(self):
        _capi.check(_capi.lib().cusat_rx_chain_reset(self._h))

    def warmup(self):
        _capi.check(_capi.lib().cusat_rx_chain_warmup(self._h))

    def update_snr(self, snr_db):
        _capi.lib().cusat_rx_chain_update_snr(self._h, snr_db)

    def set_block_when_full(self, on):
        _capi.lib().cusat_rx_chain_set_block_when_full(self._h, 1 if on else 0)

    def set_copy_threads(self, helpers):
        """Split each frame's copy into the ring across `helpers` threads."""
        _capi.check(_capi.lib().cusat_rx_chain_set_copy_threads(self._h, helpers))

    def set_decode_budget(self, budget):
        if budget is not None:
            _capi.check(_capi.lib().cusat_rx_chain_set_decode_budget(self._h, budget._h))
            self._budget = budget

    def set_weights(self, weights):
        w, n = _weights_arg(weights)
        _capi.check(_capi.lib().cusat_rx_chain_set_weights(self._h, w, n))

    def _stats(self):
        out = np.zeros(12, np.float64)
        _capi.check(_capi.lib().cusat_rx_chain_stats(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def frame_count(self):
        return int(self._stats()[0])

    def frame_error_count(self):
        return int(self._stats()[1])

    def gpu_drop_count(self):
        return int(self._stats()[2])

    def gpu_inflight(self):
        return int(self._stats()[3])

    def gpu_pending_launch(self):
        return int(self._stats()[4])

    def force_drain_count(self):
        return int(self._stats()[5])

    def pending_count(self):
        return int(self._stats()[6])

    def snr_db(self):
        return float(self._stats()[7])

    data_snr_db = snr_db

    def precision(self):
        return float(self._stats()[8])

    def noise_var(self):
        return float(self._stats()[9])

    def batch_age_s(self):
        return float(self._stats()[10])

    def batch_size(self):
        return self._batch_size

    def max_output_bytes(self):
        return self._max_out


class rx_fec_pool:
    """One rx_fec_chain per enabled MODCOD (modcod_idx values of the MODCOD
    table) behind one decode budget; output blocks in submission order.
    mixed=True: every MODCOD in one slot ring of slot_frames-frame
    multi-MODCOD launches, no wait at a MODCOD change, same output."""

    def __init__(self, framesize, enabled_modcods, max_trials=25, cuda_max_batch=64, n_gpu_streams=8,
                 micro_batch=4, mixed=False, slot_frames=64):
        from .enums import modcod_by_index
        triples = []
        for idx in enabled_modcods:
            m = modcod_by_index(int(idx))
            triples += [m[0], m[1], m[2]]
        arr = np.asarray(triples, np.int32)
        h = ctypes.c_void_p()
        if mixed:
            _capi.check(_capi.lib().cusat_rx_pool_create_mixed(framesize, arr.ctypes.data, len(enabled_modcods),
                                                               max_trials, n_gpu_streams, micro_batch, slot_frames,
                                                               ctypes.byref(h)))
        else:
            _capi.check(_capi.lib().cusat_rx_pool_create(framesize, arr.ctypes.data, len(enabled_modcods),
                                                         max_trials, cuda_max_batch, n_gpu_streams, micro_batch,
                                                         ctypes.byref(h)))
        self._h = h
        self.mixed = bool(mixed)
        self._max_out = self.max_output_bytes()
        self.modcods = [int(i) for i in enabled_modcods]

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_rx_pool_destroy(self._h)
            self._h = None

    __del__ = close

    def chain(self, modcod):
        h = _capi.lib().cusat_rx_pool_chain(self._h, modcod)
        return rx_fec_chain(0, 0, 0, _handle=ctypes.c_void_p(h)) if h else None

    def submit(self, symbols, modcod, n_symbols=None):
        a, n = _symbols(symbols)
        if n_symbols is not None:
            n = min(n, int(n_symbols))
        return _check_ready(_capi.lib().cusat_rx_pool_submit(self._h, a.ctypes.data, n, modcod))

    def get_gse_output(self, max_bytes=None):
        if max_bytes is None:
            max_bytes = self._max_out
        buf = getattr(self, "_buf", None)
        if buf is None or buf.size < max(max_bytes, 1):
            buf = self._buf = np.empty(max(max_bytes, 1), np.uint8)  # reused across calls
        n = _capi.lib().cusat_rx_pool_get_gse_output(self._h, buf.ctypes.data, max_bytes)
        if n < 0:
            _capi.check(n)
        return buf[:n].copy()

    def gse_dfl_sizes(self):
        n = _capi.lib().cusat_rx_pool_gse_dfl_sizes(self._h, None, 0)
        out = np.zeros(max(n, 1), np.int32)
        _capi.lib().cusat_rx_pool_gse_dfl_sizes(self._h, out.ctypes.data, n)
        return [int(v) for v in out[:n]]

    def drain_all_completed(self):
        return _check_ready(_capi.lib().cusat_rx_pool_drain_all_completed(self._h))

    def finish_all_pending(self):
        _capi.check(_capi.lib().cusat_rx_pool_finish_all_pending(self._h))

    def launch_stale(self, max_age_ms):
        return _check_ready(_capi.lib().cusat_rx_pool_launch_stale(self._h, float(max_age_ms)))

    def reset_all(self):
        _capi.check(_capi.lib().cusat_rx_pool_reset_all(self._h))

    def warmup_all(self):
        _capi.check(_capi.lib().cusat_rx_pool_warmup_all(self._h))

    def update_snr(self, modcod, snr_db):
        _capi.lib().cusat_rx_pool_update_snr(self._h, modcod, snr_db)

    def set_copy_threads(self, helpers):
        _capi.check(_capi.lib().cusat_rx_pool_set_copy_threads(self._h, helpers))

    def _stats(self):
        out = np.zeros(5, np.float64)
        _capi.check(_capi.lib().cusat_rx_pool_stats(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def total_frame_count(self):
        return int(self._stats()[0])

    def total_error_count(self):
        return int(self._stats()[1])

    def total_gpu_drop_count(self):
        return int(self._stats()[2])

    def max_output_bytes(self):
        return int(self._stats()[3])

    def data_snr_db(self):
        return float(self._stats()[4])

    def modcod_counters(self, modcod):
        f, e = ctypes.c_uint64(), ctypes.c_uint64()
        rc = _capi.lib().cusat_rx_pool_modcod_counters(self._h, modcod, ctypes.byref(f), ctypes.byref(e))
        if rc < 0:
            _capi.check(rc)
        return (int(f.value), int(e.value)) if rc == 1 else None
