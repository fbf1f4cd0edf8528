"""ctypes binding of the CPU oracle (test infrastructure; see oracle/fec_oracle.h).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  The product package never imports it.
"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_lib = None
_ref = None


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def lib():
    global _lib
    if _lib is None:
        import sys
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as _b  # oracle/build.py
        sys.path.pop(0)
        path = _b.build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.orc_exp_neg.restype = ctypes.c_float
        _lib.orc_exp_neg.argtypes = [ctypes.c_float]
        _lib.orc_log.restype = ctypes.c_float
        _lib.orc_log.argtypes = [ctypes.c_float]
        _lib.orc_dd_snr.restype = ctypes.c_float
        _lib.orc_demap_dmax.restype = ctypes.c_float
        _lib.orc_capped_llr_gain.restype = ctypes.c_float
        _lib.orc_capped_llr_gain.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
    return _lib


def ref():
    """The reference's own host code (oracle/_ref), or None when absent."""
    global _ref
    if _ref is None:
        import sys
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as _b
        sys.path.pop(0)
        path = None
        try:
            path = _b.build_ref()
        except Exception:
            path = None
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
        _ref.ref_dd_snr.restype = ctypes.c_float
    return _ref


def code_info(fs, rate):
    out = np.zeros(10, np.int32)
    if lib().orc_code_info(fs, rate, _p(out, ctypes.c_int32)) != 0:
        raise ValueError("unsupported code")
    keys = ["N", "K", "q", "n_steps", "k_bch", "n_bch", "t", "p", "links_total", "cnl"]
    return dict(zip(keys, (int(x) for x in out)))


def ldpc_decode(fs, rate, llr, max_trials, weights=None, nthreads=8, syn_period=1):
    info = code_info(fs, rate)
    llr = np.ascontiguousarray(llr, np.int16).reshape(-1, info["N"])
    B = llr.shape[0]
    hard = np.zeros((B, info["K"] // 8), np.uint8)
    trials = np.zeros(B, np.int32)
    w = None if weights is None else _p(np.ascontiguousarray(weights, np.int16), ctypes.c_int16)
    rc = lib().orc_ldpc_decode_period(fs, rate, _p(llr, ctypes.c_int16), B, max_trials, syn_period, w,
                                      _p(hard, ctypes.c_uint8), _p(trials, ctypes.c_int32), nthreads)
    assert rc == 0
    return hard, trials


_golden = None


def golden():
    """The reference's host-code answers (tests/golden/reference_host.json)."""
    global _golden
    if _golden is None:
        import json
        with open(os.path.join(ROOT, "tests", "golden", "reference_host.json")) as f:
            _golden = json.load(f)
    return _golden


def modcod(mod, rate, fs, llr_target=320.0):
    """Oracle-side demap parameters of a MODCOD, independent of the product:
    the reference's constellation points and interleaver columns (golden
    fixtures recorded from its host code), the frame geometry by the
    reference's rules (demapper_kernel.cu:241-247: 128APSK stuffs 6 bits and
    pads 12 symbols), the formula kind, and the loudest-bit distance dmax
    computed by the oracle (demapper_kernel.cu:216-237)."""
    from cusat_gb300 import enums as E
    name = next(m[3] for m in E.MODCODS if (m[1], m[2]) == (mod, rate))
    g = next(m for m in golden()["modcods"] if m["name"] == name and m["fs"] == fs)
    bits = g["bits"]
    n = 1 << bits
    re = np.array(g["re"], np.uint32).view(np.float32)[:n].copy()
    im = np.array(g["im"], np.uint32).view(np.float32)[:n].copy()
    fec_len = 64800 if fs == 0 else 16200
    if mod == E.MOD_128APSK:
        il = (fec_len + 6) // bits
        xfec = il + 12
    else:
        xfec = fec_len // bits
        il = xfec
    kind = 0 if mod == E.MOD_QPSK else 1 if mod == E.MOD_8PSK else 2
    dmax = float(lib().orc_demap_dmax(kind, _p(re, ctypes.c_float), _p(im, ctypes.c_float), n, bits))
    return {"n_mod": bits, "n_points": n, "fecframe_len": fec_len, "xfecframe_len": xfec,
            "interleaved_len": il, "kind": kind, "points": (re + 1j * im).astype(np.complex64),
            "col_offset": np.array(g["col"], np.uint32), "dmax": dmax, "llr_target": llr_target}


def capped_llr_gain(mi, llr_gain):
    """The oracle's gain cap for a modcod() description."""
    return float(lib().orc_capped_llr_gain(mi["dmax"], mi["llr_target"], llr_gain))


def demap_modcod(sym, mi, noise_var, llr_gain):
    """Oracle demap of a modcod() description, with the oracle's own gain cap
    applied to llr_gain (as the reference's callers do)."""
    return demap(sym, mi["xfecframe_len"], mi["interleaved_len"], mi["fecframe_len"], mi["n_mod"], mi["kind"],
                 mi["points"], mi["col_offset"], noise_var, capped_llr_gain(mi, llr_gain))


def syndrome_ok(fs, rate, llr):
    llr = np.ascontiguousarray(llr, np.int16)
    return bool(lib().orc_syndrome_ok(fs, rate, _p(llr, ctypes.c_int16)))


def ldpc_encode(fs, rate, info_bytes):
    info = code_info(fs, rate)
    info_bytes = np.ascontiguousarray(info_bytes, np.uint8).reshape(-1, info["K"] // 8)
    B = info_bytes.shape[0]
    cw = np.zeros((B, info["N"] // 8), np.uint8)
    assert lib().orc_ldpc_encode(fs, rate, _p(info_bytes, ctypes.c_uint8), _p(cw, ctypes.c_uint8), B) == 0
    return cw


def bch_generator(fs, rate):
    g = np.zeros(4, np.uint64)
    p = lib().orc_bch_generator(fs, rate, _p(g, ctypes.c_uint64))
    return g, p


def bch_encode(fs, rate, msg):
    info = code_info(fs, rate)
    msg = np.ascontiguousarray(msg, np.uint8).reshape(-1, info["k_bch"] // 8)
    B = msg.shape[0]
    cw = np.zeros((B, info["n_bch"] // 8), np.uint8)
    assert lib().orc_bch_encode(fs, rate, _p(msg, ctypes.c_uint8), _p(cw, ctypes.c_uint8), B) == 0
    return cw


def bch_check(fs, rate, cw):
    info = code_info(fs, rate)
    cw = np.ascontiguousarray(cw, np.uint8).reshape(-1, info["n_bch"] // 8)
    B = cw.shape[0]
    rem = np.zeros((B, info["p"] // 8), np.uint8)
    valid = np.zeros(B, np.int32)
    assert lib().orc_bch_check(fs, rate, _p(cw, ctypes.c_uint8), _p(rem, ctypes.c_uint8),
                               _p(valid, ctypes.c_int32), B) == 0
    return rem, valid


def demap(sym, xfec, interleaved_len, fec_len, n_mod, kind, pts, col, noise_var, llr_gain):
    sym = np.ascontiguousarray(sym, np.float32).reshape(-1, xfec * 2)
    B = sym.shape[0]
    pts = np.asarray(pts, np.complex64)
    pre = np.ascontiguousarray(pts.real, np.float32)
    pim = np.ascontiguousarray(pts.imag, np.float32)
    col = np.ascontiguousarray(np.asarray(col, np.uint32).reshape(8))
    out = np.zeros((B, fec_len), np.int16)
    assert lib().orc_demap(_p(sym, ctypes.c_float), B, xfec, interleaved_len, fec_len, n_mod, kind,
                           _p(pre, ctypes.c_float), _p(pim, ctypes.c_float), len(pts),
                           _p(col, ctypes.c_uint32), ctypes.c_float(noise_var),
                           ctypes.c_float(llr_gain), _p(out, ctypes.c_int16)) == 0
    return out


def map_symbols(cw, xfec, n_mod, col, stride, pts, interleaved_len=None, fec_len=None):
    cw = np.ascontiguousarray(cw, np.uint8)
    B = cw.shape[0]
    pts = np.asarray(pts, np.complex64)
    pre = np.ascontiguousarray(pts.real, np.float32)
    pim = np.ascontiguousarray(pts.imag, np.float32)
    col = np.ascontiguousarray(np.asarray(col, np.uint32).reshape(8))
    sym = np.zeros((B, xfec * 2), np.float32)
    il = xfec if interleaved_len is None else interleaved_len
    fl = cw.shape[1] * 8 if fec_len is None else fec_len
    assert lib().orc_map(_p(cw, ctypes.c_uint8), B, cw.shape[1], xfec, il, fl, n_mod, _p(col, ctypes.c_uint32),
                         stride, _p(pre, ctypes.c_float), _p(pim, ctypes.c_float),
                         _p(sym, ctypes.c_float)) == 0
    return sym


def bnl_update(raw, old):
    d = np.zeros(1, np.int32)
    m = lib().orc_bnl_update(raw, old, _p(d, ctypes.c_int32))
    return m, int(d[0])


def nms_train(fs, rate, llr, cw, T, theta, grad=True, dtype=np.float32, nthreads=8, iter_w=None):
    """Loss and gradient (sums over frames) of the unrolled learned min-sum
    model; theta [T, 32, 2] = {beta, alpha}; iter_w [T] loss weights or None
    (uniform).  dtype float32 or float64."""
    info = code_info(fs, rate)
    llr = np.ascontiguousarray(llr, np.int16).reshape(-1, info["N"])
    cw = np.ascontiguousarray(cw, np.uint8).reshape(-1, info["N"] // 8)
    assert llr.shape[0] == cw.shape[0]
    ct = ctypes.c_float if dtype == np.float32 else ctypes.c_double
    fn = lib().orc_nms_train_f32 if dtype == np.float32 else lib().orc_nms_train_f64
    th = np.ascontiguousarray(theta, dtype).reshape(T, 32, 2)
    g = np.zeros((T, 32, 2), dtype)
    loss = np.zeros(1, dtype)
    iw = None if iter_w is None else np.ascontiguousarray(iter_w, dtype).reshape(T)
    rc = fn(fs, rate, _p(llr, ctypes.c_int16), _p(cw, ctypes.c_uint8), llr.shape[0], T, _p(th, ct),
            None if iw is None else _p(iw, ct), _p(g, ct) if grad else None, _p(loss, ct), nthreads)
    assert rc == 0
    return float(loss[0]), g


def bb_prbs(n):
    out = np.zeros(n, np.uint8)
    lib().orc_bb_prbs(_p(out, ctypes.c_uint8), n)
    return out


def bb_extract(hard, kbch, trials, valid, max_out):
    """The RX chain's post-FEC stage over a batch: (packed data fields,
    lengths [B], offsets [B + 1])."""
    hard = np.ascontiguousarray(hard, np.uint8)
    B, stride = hard.shape
    trials = np.ascontiguousarray(trials, np.int32)
    valid = np.ascontiguousarray(valid, np.int32)
    out = np.zeros(max(max_out, 1), np.uint8)
    lengths = np.zeros(B, np.int32)
    offsets = np.zeros(B + 1, np.int32)
    assert lib().orc_bb_extract(_p(hard, ctypes.c_uint8), stride, kbch, _p(trials, ctypes.c_int32),
                                _p(valid, ctypes.c_int32), B, _p(out, ctypes.c_uint8), max_out,
                                _p(lengths, ctypes.c_int32), _p(offsets, ctypes.c_int32)) == 0
    return out[:offsets[B]], lengths, offsets


def bb_build(data, kbch, ts_gs=0):
    data = np.ascontiguousarray(data, np.uint8)
    out = np.zeros(kbch, np.uint8)
    assert lib().orc_bb_build(_p(data, ctypes.c_uint8), len(data), kbch, ts_gs, _p(out, ctypes.c_uint8)) == 0
    return out


def dd_snr(sym, pts, stride=1, qpsk=False):
    """Decision-directed SNR (linear) of float32 (re, im) symbols against
    points [2 * n_points] (ignored for QPSK)."""
    sym = np.ascontiguousarray(sym, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    return float(lib().orc_dd_snr(_p(sym, ctypes.c_float), sym.size // 2, _p(pts, ctypes.c_float),
                                  pts.size // 2, stride, 1 if qpsk else 0))


def pl_rotation(gold, n):
    """The oracle's PL scrambling rotation index R_n(i), i < n."""
    r = np.zeros(n, np.uint8)
    assert lib().orc_pl_rotation(gold, _p(r, ctypes.c_uint8), n) == 0
    return r


def pl_extract(payload, slots, pilots, r, slot_rot=None):
    """The oracle's data symbols of one PLFRAME payload ((re, im) pairs)."""
    payload = np.ascontiguousarray(payload, np.float32)
    r = np.ascontiguousarray(r, np.uint8)
    out = np.zeros(2 * 90 * slots, np.float32)
    rot = None if slot_rot is None else _p(np.ascontiguousarray(slot_rot, np.float32), ctypes.c_float)
    assert lib().orc_pl_extract(_p(payload, ctypes.c_float), slots, 1 if pilots else 0, _p(r, ctypes.c_uint8), rot,
                                _p(out, ctypes.c_float)) == 0
    return out


def pl_frame_payload(data, slots, pilots, r):
    """Test traffic for the PL receiver tail: the transmitted payload of one
    PLFRAME -- data slots with a pilot block (36 symbols (1 + j)/sqrt 2)
    after every 16 slots when pilots are on (EN 302 307-1 clause 5.5.3),
    scrambled by e^{+j R pi/2} (clause 5.5.4)."""
    data = np.asarray(data, np.float32).reshape(-1, 2)
    n_pb = (slots - 1) // 16 if pilots else 0
    a = np.float32(np.sqrt(0.5))
    rows = []
    for s in range(slots):
        rows.append(data[90 * s:90 * (s + 1)])
        if pilots and s % 16 == 15 and (s + 1) // 16 <= n_pb:
            rows.append(np.tile(np.array([[a, a]], np.float32), (36, 1)))
    pay = np.concatenate(rows)
    rr = r[:len(pay)] & 3
    re, im = pay[:, 0].copy(), pay[:, 1].copy()
    out = np.empty_like(pay)
    # e^{+j R pi/2}: 1, j, -1, -j
    out[:, 0] = np.select([rr == 0, rr == 1, rr == 2, rr == 3], [re, -im, -re, im])
    out[:, 1] = np.select([rr == 0, rr == 1, rr == 2, rr == 3], [im, re, -im, -re])
    return out.reshape(-1)


class RefGpu:
    """The reference's own demapper and layered-decoder kernels, compiled
    unchanged into oracle/_ref/*.cubin and launched through oracle/ref_gpu.c
    the way the reference's host classes launch them
    (demapper_kernel.cu:293-330, ldpc_decode_kernel.cu:991-1285).  Test
    infrastructure: it holds the reference's kernels against the oracle and
    times them beside this project's kernels on the same GPU."""

    def __init__(self):
        import sys
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as _b
        sys.path.pop(0)
        paths = _b.ref_cubin_paths()
        missing = [p for p in paths.values() if not os.path.exists(p)]
        if missing:
            raise FileNotFoundError(f"reference cubins not built: {missing}")
        so = _b.build_ref_gpu()
        if so is None:
            raise FileNotFoundError("cuda.h not found: oracle/ref_gpu.c not built")
        L = ctypes.CDLL(so)
        L.rg_last_error.restype = ctypes.c_char_p
        L.rg_dec_create.restype = ctypes.c_void_p
        L.rg_dec_create.argtypes = [ctypes.c_int] * 4
        L.rg_dec_destroy.argtypes = [ctypes.c_void_p]
        L.rg_dec_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_dec_launch.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                                    ctypes.c_uint64, ctypes.c_void_p]
        L.rg_demap_launch.argtypes = [ctypes.c_uint64] * 4 + [ctypes.c_int] * 5 + [
            ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]
        self.L = L
        self._check(L.rg_open(paths["ref_ldpc_decode.sm_103.cubin"].encode(),
                              paths["ref_demap.sm_103.cubin"].encode()))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.L.rg_last_error().decode())

    def decoder(self, fs, rate, max_trials, max_batch):
        return RefGpuDecoder(self, fs, rate, max_trials, max_batch)

    def demap(self, sym_dev, out_dev, pts_re_dev, pts_im_dev, mi, noise_var, llr_gain, B, stream):
        """demap_deinterleave_kernel of B frames; llr_gain already capped.
        QPSK and 8PSK get no point table, as demapper_cuda uploads one only
        for 8APSK and the 16+ point families (demapper_kernel.cu:252-262):
        its 8PSK formula branch is taken only without a table (:76)."""
        col = np.ascontiguousarray(mi["col_offset"], np.uint32)
        table = mi["kind"] == 2
        re_p = pts_re_dev.data_ptr() if table else 0
        im_p = pts_im_dev.data_ptr() if table else 0
        self._check(self.L.rg_demap_launch(sym_dev.data_ptr(), out_dev.data_ptr(), re_p,
                                           im_p, mi["xfecframe_len"], mi["interleaved_len"],
                                           mi["fecframe_len"], mi["n_mod"], mi["n_points"], col.ctypes.data,
                                           noise_var, llr_gain, B, stream.cuda_stream))


class RefGpuDecoder:
    def __init__(self, rg, fs, rate, max_trials, max_batch):
        self.rg = rg
        h = rg.L.rg_dec_create(fs, rate, max_trials, max_batch)
        if not h:
            raise RuntimeError(rg.L.rg_last_error().decode())
        self.h = h
        info = np.zeros(8, np.int32)
        rg.L.rg_dec_info(h, info.ctypes.data)
        self.N, self.K, self.R, self.q, self.cnl, self.lt_alloc, self.n_steps, self.smem = (int(v) for v in info)

    def launch(self, llr_dev, B, hard_dev, result_dev, stream):
        self.rg._check(self.rg.L.rg_dec_launch(self.h, llr_dev.data_ptr(), B, hard_dev.data_ptr(),
                                               result_dev.data_ptr(), stream.cuda_stream))

    def close(self):
        if self.h:
            self.rg.L.rg_dec_destroy(self.h)
            self.h = None
