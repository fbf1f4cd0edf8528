"""The CPU oracle against the known answers of the reference's own tests.

Runs without a GPU.  Each test names the reference test it restates.
"""
import numpy as np
import pytest

import oracle_lib as O

NORMAL, SHORT = 0, 1
RATES_NORMAL = list(range(11))  # RATE_1_4 .. RATE_9_10


def test_message_update_known_answers():
    # lib/qa_ldpc_message_update.cc:10-27
    assert O.bnl_update(300, 127) == (127, 0)
    assert O.bnl_update(300, -127) == (127, 254)
    assert O.bnl_update(-300, 127) == (-127, -254)
    assert O.bnl_update(42, -5) == (42, 47)


def _coeffs(g):
    return [i for i in range(256) if (int(g[i // 64]) >> (i % 64)) & 1]


def test_bch_generator_degrees_and_field_polynomials():
    # lib/qa_bch_code.cc:34-57
    assert O.bch_generator(NORMAL, 0)[1] == 192      # n 16200, t 12
    assert O.bch_generator(NORMAL, 6)[1] == 192      # 3/4: t 12
    assert O.bch_generator(NORMAL, 5)[1] == 160      # 2/3: t 10
    assert O.bch_generator(NORMAL, 9)[1] == 128      # 8/9: t 8
    assert O.bch_generator(SHORT, 0)[1] == 168
    assert O.code_info(NORMAL, 0)["k_bch"] == 16008
    # g1 is the field polynomial: product of one factor = first minimal polynomial
    g, p = O.bch_generator(NORMAL, 9)  # t = 8: g1..g8; check g1 through the data instead
    from_data = [0x1002D, 0x402B]
    assert [i for i in range(17) if (from_data[0] >> i) & 1] == [0, 2, 3, 5, 16]
    assert [i for i in range(15) if (from_data[1] >> i) & 1] == [0, 1, 3, 5, 14]


def _bitserial_rem(cw_bytes, g, p):
    """qa_bch_code.cc:17-32: remainder of the big-endian bit string mod g."""
    r = [0] * p
    for byte in cw_bytes:
        for b in range(7, -1, -1):
            top = r[p - 1]
            r = [(int(byte) >> b) & 1] + r[:-1]
            if top:
                r = [r[i] ^ ((int(g[i // 64]) >> (i % 64)) & 1) for i in range(p)]
    return r


@pytest.mark.parametrize("fs,rate", [(NORMAL, 0), (NORMAL, 10), (SHORT, 9)])
def test_bch_codewords_are_multiples_of_g(fs, rate):
    # qa_bch_code.cc:59-78 (independent bit-serial remainder)
    rng = np.random.default_rng(1)
    ci = O.code_info(fs, rate)
    msg = rng.integers(0, 256, (2, ci["k_bch"] // 8), dtype=np.uint8)
    cw = O.bch_encode(fs, rate, msg)
    assert (cw[:, :ci["k_bch"] // 8] == msg).all()  # systematic
    g, p = O.bch_generator(fs, rate)
    assert not any(_bitserial_rem(cw[0], g, p))
    rem, valid = O.bch_check(fs, rate, cw)
    assert valid.all() and not rem.any()


def test_bch_linearity():
    # qa_bch_code.cc:80-97
    rng = np.random.default_rng(2)
    ci = O.code_info(SHORT, 3)
    a = rng.integers(0, 256, ci["k_bch"] // 8, dtype=np.uint8)
    b = rng.integers(0, 256, ci["k_bch"] // 8, dtype=np.uint8)
    ca, cb, cab = (O.bch_encode(SHORT, 3, x)[0] for x in (a, b, a ^ b))
    assert (cab == (ca ^ cb)).all()


@pytest.mark.parametrize("fs,rate", [(NORMAL, 4), (NORMAL, 5), (NORMAL, 9), (SHORT, 3)])
def test_bch_single_bit_corruption_detected(fs, rate):
    # apps/bench_bch_gpu.cc:87-104: positions {0, k-1, k, n-1}, frames f % 3 != 1
    ci = O.code_info(fs, rate)
    k, n = ci["k_bch"] // 8, ci["n_bch"] // 8
    rng = np.random.default_rng(ci["n_bch"])
    cw = O.bch_encode(fs, rate, rng.integers(0, 256, (7, k), dtype=np.uint8))
    for pos in (0, k - 1, k, n - 1):
        bad = cw.copy()
        for f in range(7):
            if f % 3 != 1:
                bad[f, pos] ^= 1 << (f % 8)
        _, valid = O.bch_check(fs, rate, bad)
        assert list(valid) == [int(f % 3 == 1) for f in range(7)]


@pytest.mark.parametrize("rate", RATES_NORMAL)
def test_noiseless_roundtrip_all_normal_rates(rate):
    # lib/qa_ldpc_encode.cc:35-87: seed 42, +-127 LLRs, 50 trials
    ci = O.code_info(NORMAL, rate)
    rng = np.random.default_rng(42)
    info = rng.integers(0, 256, (1, ci["K"] // 8), dtype=np.uint8)
    cw = O.ldpc_encode(NORMAL, rate, info)
    assert (cw[:, :ci["K"] // 8] == info).all()
    llr = np.where(np.unpackbits(cw, axis=1) == 1, -127, 127).astype(np.int16)
    assert O.syndrome_ok(NORMAL, rate, llr[0])
    hard, trials = O.ldpc_decode(NORMAL, rate, llr, 50)
    assert trials[0] > 0 and (hard == info).all()


@pytest.mark.parametrize("rate", range(10))
def test_noiseless_roundtrip_short_rates(rate):
    ci = O.code_info(SHORT, rate)
    rng = np.random.default_rng(7)
    info = rng.integers(0, 256, (1, ci["K"] // 8), dtype=np.uint8)
    cw = O.ldpc_encode(SHORT, rate, info)
    llr = np.where(np.unpackbits(cw, axis=1) == 1, -127, 127).astype(np.int16)
    hard, trials = O.ldpc_decode(SHORT, rate, llr, 50)
    assert trials[0] == 50 and (hard == info).all()


def test_decoder_corrects_errors_and_reports_failure():
    # a codeword with a handful of flipped LLRs converges in a few iterations;
    # random LLRs do not converge (trials = -1) and still return hard bits
    ci = O.code_info(SHORT, 3)
    rng = np.random.default_rng(3)
    info = rng.integers(0, 256, (1, ci["K"] // 8), dtype=np.uint8)
    cw = O.ldpc_encode(SHORT, 3, info)
    llr = np.where(np.unpackbits(cw, axis=1) == 1, -40, 40).astype(np.int16)
    flip = rng.choice(ci["N"], 30, replace=False)
    llr[0, flip] = -llr[0, flip] // 4
    hard, trials = O.ldpc_decode(SHORT, 3, llr, 50)
    assert 0 < trials[0] < 50 and (hard == info).all()
    junk = rng.integers(-20, 20, (1, ci["N"]), dtype=np.int16)
    hard, trials = O.ldpc_decode(SHORT, 3, junk, 5)
    assert trials[0] == -1 and hard.shape == (1, ci["K"] // 8)


def test_zero_iterations():
    ci = O.code_info(SHORT, 3)
    llr = np.full((1, ci["N"]), 5, np.int16)  # all-zero word is a codeword
    hard, trials = O.ldpc_decode(SHORT, 3, llr, 0)
    assert trials[0] == 0 and not hard.any()
    llr[0, 0] = -5
    _, trials = O.ldpc_decode(SHORT, 3, llr, 0)
    assert trials[0] == -1


def test_exp_log_accuracy():
    xs = np.linspace(0, 16, 2001, dtype=np.float32)
    e = np.array([O.lib().orc_exp_neg(float(x)) for x in xs])
    assert np.max(np.abs(e - np.exp(-xs.astype(np.float64))) / np.exp(-xs.astype(np.float64))) < 2e-6
    ys = np.float32(10.0) ** np.linspace(-30, 2, 997, dtype=np.float32)
    l = np.array([O.lib().orc_log(float(y)) for y in ys])
    assert np.max(np.abs(l - np.log(ys.astype(np.float64)))) < 2e-5
