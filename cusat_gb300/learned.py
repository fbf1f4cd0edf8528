"""Learned min-sum weights: training, quantisation, persistence, FER.

The weights are one {beta, alpha} pair per decoding iteration and check
degree.  They are trained in FP32 on the GPU by this library's unrolled
forward/backward kernels (cusat_nms_train_step) on frames generated by this
package's BCH/LDPC encoder, mapper, an AWGN channel and the library's soft
demapper; then quantised into the integer decoder's table (beta in LLR
units, alpha in 64ths; cusat_*_set_weights).  The plain offset min-sum
decoder (beta 1, no scaling) stays the fallback: a MODCOD without a weight
file decodes plain.

The reference has no learned decoder; its normalised-min-sum hook
(ldpc_decode_kernel.cu:75-90, alpha in 64ths, odd-symmetric rounding) is the
integer form used here.
"""
import ctypes
import json
import os

import numpy as np

from . import _capi, code_info
from .enums import find_modcod

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


class nms_trainer:
    """The FP32 unrolled model of one code on the GPU (forward + backward)."""

    def __init__(self, framesize, rate, n_iter, max_batch):
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().cusat_nms_trainer_create(framesize, rate, n_iter, max_batch, ctypes.byref(h)))
        self._h = h
        out = (ctypes.c_int32 * 6)()
        _capi.check(_capi.lib().cusat_nms_trainer_info(h, out))
        self.n_ldpc, self.k_ldpc, self.n_iter, self.max_batch, self.deg_lo, self.deg_hi = list(out)
        cnt = (ctypes.c_int32 * 32)()
        _capi.check(_capi.lib().cusat_nms_trainer_degree_counts(h, cnt))
        self.degree_counts = list(cnt)

    def tied_degrees(self):
        """{rare degree: degree it follows}: a degree with fewer checks than
        one layer (check 0 of layer 0, which lacks the wrap edge) gets a
        gradient from a handful of checks per frame; training ties it to the
        next degree up instead of letting that noise steer it."""
        out = {}
        for d, n in enumerate(self.degree_counts):
            if 0 < n < 360:
                up = next((e for e in range(d + 1, 32) if self.degree_counts[e] >= 360), None)
                if up is not None:
                    out[d] = up
        return out

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().cusat_nms_trainer_destroy(self._h)
            self._h = None

    __del__ = close

    def step(self, llr, cw, batch, theta, grad, loss, stream=None, iter_w=None):
        """Adds the summed loss (and gradient, unless grad is None) of `batch`
        frames; all arguments are device tensors or addresses; iter_w: loss
        weight per iteration (device) or None (uniform)."""
        from . import _addr, _stream
        _capi.check(_capi.lib().cusat_nms_train_step(self._h, _addr(llr), _addr(cw), batch, _addr(theta),
                                                     _addr(iter_w), _addr(grad), _addr(loss), _stream(stream)))


def plain_theta(n_iter):
    """{beta, alpha} of the plain offset min-sum decoder for every entry."""
    th = np.zeros((n_iter, 32, 2), np.float32)
    th[:, :, 0] = 1.0
    th[:, :, 1] = 1.0
    return th


def quantize(theta):
    """FP32 {beta, alpha} -> the integer decoder's {beta, alpha in 64ths}."""
    th = np.asarray(theta, np.float32)
    w = np.zeros(th.shape, np.int16)
    w[..., 0] = np.clip(np.rint(th[..., 0]), 0, 127)
    w[..., 1] = np.clip(np.rint(th[..., 1] * 64.0), 1, 255)
    return w


def dequantize(w):
    w = np.asarray(w)
    th = np.zeros(w.shape, np.float32)
    th[..., 0] = w[..., 0]
    th[..., 1] = np.where(w[..., 1] > 0, w[..., 1] / 64.0, 1.0)
    return th


def weights_path(name, framesize):
    return os.path.join(WEIGHTS_DIR, f"{name.replace('/', '_')}_{'short' if framesize == 1 else 'normal'}.json")


def save_weights(path, name, framesize, w, meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    w = np.asarray(w, np.int16)
    doc = {"modcod": name, "framesize": int(framesize), "n_iter": int(w.shape[0]),
           "layout": "[n_iter][32 check degrees][beta, alpha/64]", "weights": w.tolist(), "meta": meta}
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


def load_weights(name, framesize, path=None, adopted_only=True):
    """The stored int16 table [n_iter, 32, 2], or None (decode plain): a
    weight file that was not adopted (its learned FER lost to the plain
    decoder somewhere on its grid) is ignored unless adopted_only is False."""
    path = path or weights_path(name, framesize)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        doc = json.load(f)
    if adopted_only and not doc.get("meta", {}).get("adopted", False):
        return None
    return np.asarray(doc["weights"], np.int16)


def adopted(rows, learned_key, plain_key):
    """True when, at every Es/N0 of the table, the learned decoder's frame
    errors do not exceed the plain decoder's by more than chance: learned
    FER <= 1.5 x plain FER + 3 / frames."""
    for r in rows:
        a, b = r[learned_key], r[plain_key]
        if a["fer"] > 1.5 * b["fer"] + 3.0 / max(a["frames"], 1):
            return False
    return True


class ChannelPool:
    """Noisy frames of one MODCOD made on the GPU: fresh random messages,
    BCH + LDPC encoded and mapped by the library's generator (unit average
    symbol energy), AWGN per frame (N0 = 1/SNR, sigma = sqrt(N0/2) per
    component), demapped by the library's demapper with llr_gain =
    min(4/N0, 1000) capped like the chain (the conventions of the reference's
    apps/bench_coded_modulation.cc:287-308,373-391)."""

    def __init__(self, name, framesize, n_codewords, seed, max_batch, torch):
        """n_codewords is kept for callers; every draw encodes fresh messages."""
        from . import demapper_cuda, generator
        self.torch = torch
        _, self.mod, self.rate, _, _, self.threshold = find_modcod(name)
        self.fs = framesize
        ci = code_info(framesize, self.rate)
        self.n, self.k_bch = ci["n_ldpc"], ci["k_bch"]
        self.gen_tx = generator(self.mod, self.rate, framesize, max_batch)
        self.dm = demapper_cuda(self.mod, self.rate, framesize, max_batch)
        self.max_batch = max_batch
        self.gen = torch.Generator(device="cuda")
        self.gen.manual_seed(seed)

    def draw(self, batch, esn0_db, stream=None):
        """(noisy symbols, int16 LLRs, codewords, N0, gain) of `batch` fresh
        frames, device tensors."""
        torch = self.torch
        st = stream or torch.cuda.current_stream()
        n0 = float(np.float32(1.0 / 10 ** (esn0_db / 10.0)))
        sigma = float(np.sqrt(n0 / 2.0))
        msg = torch.randint(0, 256, (batch, self.gen_tx.msg_bytes), dtype=torch.uint8, device="cuda",
                            generator=self.gen)
        cw = torch.empty((batch, self.gen_tx.cw_bytes), dtype=torch.uint8, device="cuda")
        sym = torch.empty((batch, 2 * self.gen_tx.xfec), dtype=torch.float32, device="cuda")
        self.gen_tx.generate(msg, batch, cw, sym, st)
        sym += sigma * torch.randn(sym.shape, device="cuda", generator=self.gen)
        llr = torch.empty((batch, self.n), dtype=torch.int16, device="cuda")
        gain = min(4.0 / n0, 1000.0)
        # the receive chain caps the gain the same way (demapper_kernel.cu:283-291)
        self.dm.demap_launch(sym, batch, n0, self.dm.capped_llr_gain(gain), llr, st)
        return sym, llr, cw, n0, gain


def train(name, framesize, n_iter=20, esn0_grid=None, n_frames=100000, batch=128, lr=0.02, seed=1,
          n_codewords=256, log_every=0, log=print, beta_lr_scale=1.0, lr_min_frac=0.1, theta0=None,
          iter_weights=None):
    """Trains {beta, alpha}[n_iter][degree] for one MODCOD with Adam (step
    lr for alpha, lr * beta_lr_scale for beta, cosine decay to lr_min_frac);
    returns (theta float32 [n_iter, 32, 2], history of (frames, mean loss)).
    iter_weights: loss weight of each iteration (default uniform)."""
    import torch
    thr = find_modcod(name)[5]
    if esn0_grid is None:
        esn0_grid = [thr - 0.5 + 0.25 * k for k in range(7)]
    pool = ChannelPool(name, framesize, n_codewords, seed, batch, torch)
    tr = nms_trainer(framesize, pool.rate, n_iter, batch)
    th0 = plain_theta(n_iter) if theta0 is None else np.asarray(theta0, np.float32)
    theta = torch.from_numpy(np.ascontiguousarray(th0)).cuda()
    scale = torch.ones_like(theta)
    scale[:, :, 0] = beta_lr_scale
    grad = torch.zeros_like(theta)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    iw = None
    if iter_weights is not None:
        iw = torch.tensor(np.asarray(iter_weights, np.float32).reshape(n_iter), device="cuda")
    m = torch.zeros_like(theta)
    v = torch.zeros_like(theta)
    b1, b2, eps = 0.9, 0.999, 1e-8
    ties = tr.tied_degrees()
    used = torch.tensor([n > 0 and d not in ties for d, n in enumerate(tr.degree_counts)])
    mask = used.cuda().view(1, 32, 1).expand_as(theta).float()
    history, acc, acc_n = [], 0.0, 0
    steps = max(1, n_frames // batch)
    for k in range(steps):
        esn0 = esn0_grid[k % len(esn0_grid)]
        _, llr, cw, _, _ = pool.draw(batch, esn0)
        grad.zero_()
        loss.zero_()
        tr.step(llr, cw, batch, theta, grad, loss, iter_w=iw)
        g = grad * mask / batch
        m.mul_(b1).add_(g, alpha=1 - b1)
        v.mul_(b2).addcmul_(g, g, value=1 - b2)
        mh = m / (1 - b1 ** (k + 1))
        vh = v / (1 - b2 ** (k + 1))
        lr_k = lr * (lr_min_frac + (1 - lr_min_frac) * 0.5 * (1 + np.cos(np.pi * k / steps)))
        theta.sub_(lr_k * scale * mh / (vh.sqrt() + eps))
        theta[:, :, 0].clamp_(0.0, 127.0)
        theta[:, :, 1].clamp_(1.0 / 64.0, 2.0)
        for d, up in ties.items():
            theta[:, d, :] = theta[:, up, :]
        acc += float(loss.item()) / batch
        acc_n += 1
        if log_every and (k + 1) % log_every == 0:
            history.append(((k + 1) * batch, acc / acc_n))
            if log:
                log(f"{name} frames {(k + 1) * batch} loss {acc / acc_n:.5f}")
            acc, acc_n = 0.0, 0
    if acc_n:
        history.append((steps * batch, acc / acc_n))
    return theta.cpu().numpy(), history


def frame_errors(name, framesize, esn0_db, n_iter, weights, n_frames, batch=256, seed=7, min_errors=None,
                 stream=None):
    """Frame error rate of the integer decoder (receive chain) with `weights`
    (None = plain) at `n_iter` maximum iterations on fresh noisy frames.
    A frame is in error when its decoded k_ldpc bits differ from the sent
    ones.  Stops early after `min_errors` frame errors.  Returns a dict."""
    import torch
    from . import rx_fec
    pool = ChannelPool(name, framesize, 256, seed, batch, torch)
    rx = rx_fec(pool.mod, pool.rate, framesize, n_iter, batch)
    rx.set_weights(weights)
    kb = rx.k_bytes
    hard = torch.zeros((batch, kb), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(batch, dtype=torch.int32, device="cuda")
    frames = errors = fails = 0
    iters = 0
    st = stream or torch.cuda.current_stream()
    while frames < n_frames:
        b = min(batch, n_frames - frames)
        sym, _, cw, n0, gain = pool.draw(b, esn0_db, st)
        rx.launch(sym, b, n0, gain, hard, trials, None, st)
        bad = (hard[:b] != cw[:, :kb]).any(dim=1)
        t = trials[:b]
        errors += int(bad.sum().item())
        fails += int((t < 0).sum().item())
        iters += int(torch.where(t >= 0, n_iter - t, torch.full_like(t, n_iter)).sum().item())
        frames += b
        if min_errors and errors >= min_errors:
            break
    return {"esn0_db": esn0_db, "frames": frames, "frame_errors": errors, "fer": errors / frames,
            "decoder_failures": fails, "mean_iterations": iters / frames}


def fer_table(name, framesize, esn0_list, decoders, min_errors=200, max_frames=1000000, batch=256, seed=7,
              log=None):
    """FER rows: for every Es/N0 and (label, n_iter, weights) decoder, frames
    until min_errors frame errors or max_frames frames."""
    rows = []
    for es in esn0_list:
        row = {"esn0_db": round(float(es), 3)}
        for label, n_iter, w in decoders:
            r = frame_errors(name, framesize, es, n_iter, w, n_frames=max_frames, batch=batch, seed=seed,
                             min_errors=min_errors)
            row[label] = {k: r[k] for k in ("fer", "frame_errors", "frames", "mean_iterations")}
        rows.append(row)
        if log:
            log(json.dumps(row))
    return rows


def main(argv=None):
    """python -m cusat_gb300.learned --modcod qpsk1/3 [--short] --frames 1000000
    trains the weights on the GPU, measures FER (learned at --iters vs plain at
    --iters and --plain-iters) on the threshold grid and writes the weight
    file with the FER table, marked adopted when the learned decoder's FER is
    nowhere worse than the plain decoder's at --plain-iters (load_weights
    ignores files that are not)."""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--modcod", required=True)
    ap.add_argument("--short", action="store_true")
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--plain-iters", type=int, default=50)
    ap.add_argument("--frames", type=int, default=1000000)
    ap.add_argument("--batch", type=int, default=128)
    ap.add_argument("--lr", type=float, default=0.02)
    ap.add_argument("--beta-lr-scale", type=float, default=1.0)
    ap.add_argument("--loss", choices=["uniform", "last"], default="uniform")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fer-frames", type=int, default=1000000)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    fs = 1 if args.short else 0
    T = args.iters
    thr = find_modcod(args.modcod)[5]
    grid = [thr - 0.5 + 0.25 * k for k in range(7)]
    iw = None if args.loss == "uniform" else [0.0] * (T - 1) + [1.0]
    t0 = time.time()
    theta, hist = train(args.modcod, fs, n_iter=T, esn0_grid=grid, n_frames=args.frames, batch=args.batch,
                        lr=args.lr, seed=args.seed, beta_lr_scale=args.beta_lr_scale, iter_weights=iw,
                        log_every=max(1, args.frames // args.batch // 20))
    train_s = time.time() - t0
    w = quantize(theta)
    rows = fer_table(args.modcod, fs, grid, [("plain%d" % args.plain_iters, args.plain_iters, None),
                                              ("plain%d" % T, T, None), ("learned%d" % T, T, w)],
                     max_frames=args.fer_frames, log=print)
    ok = adopted(rows, "learned%d" % T, "plain%d" % args.plain_iters)
    meta = {"adopted": ok, "train": {"frames": args.frames, "batch": args.batch, "lr": args.lr, "beta_lr_scale": args.beta_lr_scale,
                      "loss": args.loss, "esn0_grid_db": [round(g, 3) for g in grid], "seconds": round(train_s, 1),
                      "loss_history": [[int(a), float(b)] for a, b in hist], "seed": args.seed},
            "fer": rows, "fer_rule": "200 frame errors or %d frames per point" % args.fer_frames}
    path = args.out or weights_path(args.modcod, fs)
    save_weights(path, args.modcod, fs, w, meta)
    print("wrote", path)


if __name__ == "__main__":
    main()
