"""Host side of the learned weights: quantisation, the weight files and the
adoption rule (no GPU)."""
import json

import numpy as np

from cusat_gb300 import learned
from cusat_gb300 import enums as E


def test_quantize_round_trip_and_limits():
    th = learned.plain_theta(4)
    w = learned.quantize(th)
    assert (w[..., 0] == 1).all() and (w[..., 1] == 64).all()
    assert np.allclose(learned.dequantize(w), th)
    th[0, 5] = (-3.0, 9.0)   # clipped to beta >= 0, alpha <= 255/64
    th[1, 5] = (500.0, 0.0)  # beta <= 127, alpha >= 1/64
    w = learned.quantize(th)
    assert tuple(w[0, 5]) == (0, 255) and tuple(w[1, 5]) == (127, 1)


def test_weight_files():
    w = learned.load_weights("qpsk1/3", E.FECFRAME_NORMAL)
    assert w.dtype == np.int16 and w.shape == (20, 32, 2)
    assert (w[..., 0] >= 0).all() and (w[..., 0] <= 127).all() and (w[..., 1] <= 255).all()
    doc = json.load(open(learned.weights_path("qpsk1/3", E.FECFRAME_NORMAL)))
    assert doc["meta"]["adopted"] and doc["meta"]["train"]["frames"] >= 1000000
    rows = doc["meta"]["fer"]
    assert learned.adopted(rows, "learned20", "plain50")
    # every Es/N0 of the grid: at least 200 frame errors or 1e6 frames per decoder
    for r in rows:
        for k in ("plain50", "plain20", "learned20"):
            assert r[k]["frame_errors"] >= 200 or r[k]["frames"] >= 1000000
    assert learned.load_weights("16apsk3/4", E.FECFRAME_NORMAL) is None    # not adopted
    assert learned.load_weights("32apsk3/4", E.FECFRAME_NORMAL) is None    # no file


def test_every_weight_file_is_consistent():
    """Each stored table: right shape and ranges, its FER table present, and
    its adoption flag what the adoption rule says."""
    import glob
    import os
    files = glob.glob(os.path.join(learned.WEIGHTS_DIR, "*.json"))
    assert len(files) >= 2
    for f in files:
        doc = json.load(open(f))
        w = np.asarray(doc["weights"])
        assert w.shape == (doc["n_iter"], 32, 2)
        assert (w[..., 0] >= 0).all() and (w[..., 0] <= 127).all() and (w[..., 1] <= 255).all()
        assert learned.weights_path(doc["modcod"], doc["framesize"]) == f
        rows = doc["meta"]["fer"]
        assert doc["meta"]["adopted"] == learned.adopted(rows, "learned%d" % doc["n_iter"], "plain50")


def test_adoption_rule():
    row = lambda fl, fp, n=1000: {"learned20": {"fer": fl, "frames": n}, "plain50": {"fer": fp, "frames": n}}
    assert learned.adopted([row(0.0, 0.0), row(0.01, 0.5)], "learned20", "plain50")
    assert learned.adopted([row(0.002, 0.0)], "learned20", "plain50")          # within chance
    assert not learned.adopted([row(0.3, 0.01)], "learned20", "plain50")
