"""Reference-format state and estimator files, and checkpoint/resume.

The state text is checked byte for byte against the oracle's writer, which
formats it with C++ iostreams (setprecision(16), operator<< on int and
uint32) as the reference's saveState does; the reader is checked by round
trips and by loadState's two branches (same slice count, classical state).
GPU tests: the plain form's generator state matches the oracle MT19937 after
the same moves, and a run resumed from a state file continues the
uninterrupted run (plain form) or reproduces it bit for bit (walkers, whose
FP32 positions survive the 16-digit text exactly).
"""
import os

import numpy as np
import pytest

from pimc_gb300 import state as S
from pimc_gb300 import worldlines as wl


def _cfg(m=6, ne=5, seed=3, holes=False):
    rng = np.random.default_rng(seed)
    pos = (rng.random((m, ne, 3)) - 0.5) * 7.3
    pos[0, 0] = (0.0, -0.0, 1e-5)
    pos[1, 1] = (123456.78901234567, -1e-300, 5e22)
    t = np.arange(m)[:, None]
    p = np.arange(ne)[None, :]
    nxt = np.stack(np.broadcast_arrays((t + 1) % m, p), axis=-1).astype(np.int32)
    prv = np.stack(np.broadcast_arrays((t - 1) % m, p), axis=-1).astype(np.int32)
    on = np.ones((m, ne), dtype=np.uint8)
    if holes:
        on[:, 1] = 0
        nxt[:, 1] = -1
        prv[:, 1] = -1
    return dict(pos=pos, next=nxt, prev=prv, on=on)


def _words(seed=9):
    return np.random.default_rng(seed).integers(0, 2 ** 32, 625, dtype=np.uint64).astype(np.uint32)


def test_state_text_matches_cpp_streams(oracle_lib):
    for holes in (False, True):
        cfg = _cfg(holes=holes)
        words = _words()
        moves = [(12, 40), (0, 0), (7, 9)]
        ests = [(100, 3)]
        py = S.format_state(cfg, words, moves, ests)
        total = (sum(a for a, _ in moves), sum(b for _, b in moves))
        cpp = oracle_lib.format_state(cfg, words, [total] + moves + ests)
        assert py == cpp


def test_state_round_trip():
    cfg = _cfg()
    words = _words(4)
    text = S.format_state(cfg, words, [(1, 2)], [(3, 4)])
    st = S.parse_state(text)
    assert st["num_worldlines"] == 5
    assert st["counts"] == [(1, 2), (1, 2), (3, 4)]
    expect = np.vectorize(lambda x: float("%.16g" % x))(cfg["pos"])
    assert np.array_equal(st["beads"], expect)
    assert np.array_equal(st["next"], cfg["next"]) and np.array_equal(st["prev"], cfg["prev"])
    assert np.array_equal(st["worm_beads"], cfg["on"])
    assert np.array_equal(st["rng"], words)
    # FP32 values survive the 16-digit text exactly
    f32 = cfg["pos"].astype(np.float32).astype(np.float64)
    st2 = S.parse_state(S.format_state(dict(cfg, pos=f32), words))
    assert np.array_equal(st2["beads"].astype(np.float32).astype(np.float64), f32)


def test_load_state_same_slices_puts_inside():
    m, ne, side = 6, 5, 7.3
    cfg = _cfg(m, ne)
    cfg["pos"][2, 3] = (4.0, -3.9, 11.0)          # outside the box
    text = S.format_state(cfg, _words())
    got, rng = S.load_state(text, m, side)
    assert rng is not None and len(rng) == 625
    assert np.all(np.abs(got["pos"]) <= side / 2 + 1e-12)
    assert np.allclose(got["pos"][2, 3], wl.put_in_bc(np.array([4.0, -3.9, 11.0]), side))
    _, none = S.load_state(text, m, side, restart=False)
    assert none is None


def test_load_state_classical_branch():
    """loadClassicalState: a file with a different slice count gives one
    classical worldline per active slice-0 bead, packed to the left."""
    cfg = _cfg(4, 5, holes=True)
    text = S.format_state(cfg, _words())
    got, _ = S.load_state(text, 8, 100.0)
    on = got["on"]
    assert on.shape == (8, 5)
    assert np.all(on[:, :4] == 1) and np.all(on[:, 4] == 0)
    src = [0, 2, 3, 4]
    r16 = np.vectorize(lambda x: float("%.16g" % x))
    for k, n in enumerate(src):
        assert np.array_equal(got["pos"][:, k], np.broadcast_to(r16(cfg["pos"][0, n]), (8, 3)))
    assert np.all(got["next"][:, 4] == -1) and np.all(got["prev"][:, 4] == -1)
    assert np.array_equal(got["next"][7, 0], (0, 0)) and np.array_equal(got["prev"][0, 2], (7, 2))


def test_left_pack_relinks():
    cfg = _cfg(4, 4)
    # slice 2 holds only particles 0 and 3: bead (2,3) moves to (2,1) and its
    # neighbours (1,3) and (3,3) are relinked to it
    cfg["on"][2, 1] = cfg["on"][2, 2] = 0
    packed = S.left_pack(cfg)
    assert list(packed["on"][2]) == [1, 1, 0, 0]
    assert np.array_equal(packed["pos"][2, 1], cfg["pos"][2, 3])
    assert np.array_equal(packed["next"][1, 3], (2, 1))
    assert np.array_equal(packed["prev"][3, 3], (2, 1))
    assert np.array_equal(packed["next"][2, 1], (3, 3))
    assert np.array_equal(packed["prev"][2, 1], (1, 3))
    assert np.all(packed["next"][2, 3] == -1) and np.all(packed["prev"][2, 3] == -1)
    assert np.array_equal(cfg["on"][2], [1, 0, 0, 1])            # input untouched


def test_mt_save_load_resumes_stream(oracle_lib):
    a = oracle_lib.MT(123)
    for _ in range(1000):
        a.randint()
    words = a.save()
    assert words[624] == 624 - 1000 % 624
    b = oracle_lib.MT(1)
    b.load(words)
    assert [a.randint() for _ in range(700)] == [b.randint() for _ in range(700)]


def test_walker_rng_words_are_an_mtrand_image(oracle_lib):
    """left = 0 with unreloaded words: the next draw reloads first, the
    stream of MTRand(seed') from its first word."""
    words = S._walker_rng_words(5, 3, 100)
    mt = oracle_lib.MT(1)
    mt.load(words)
    ref = oracle_lib.MT(int(words[0]))
    assert [mt.randint() for _ in range(1300)] == [ref.randint() for _ in range(1300)]


def test_estimator_headers_and_rows(tmp_path):
    h = S.commented(S.scalar_header(S.ENERGY_LABELS))
    assert h.startswith("#") and len(h) == 16 * 9 and h.endswith("E/N")
    sh = S.superfluid_header()
    assert len(sh) == 16 * 26 and sh.startswith("#      rho_s/rho") and "P(-10)" in sh and "P(+0)" in sh
    ph = S.pair_correlation_header(10.0)
    assert len(ph) == 16 * 50 and ph.startswith("#      0.000E+00")
    assert S.permutation_header().split()[-1] == "40"
    qh = S.q_header([[1.0, 0.0, -0.5], [0.0, 2.0, 0.0]])
    assert qh.splitlines()[0] == ("# ESTINF: num_q = 2; (+1.00000000E+00,+0.00000000E+00,"
                                  "-5.00000000E-01) (+0.00000000E+00,+2.00000000E+00,+0.00000000E+00) ")
    assert qh.splitlines()[1] == "#%15d%16d" % (0, 1)
    assert S.format_row([1.0, -2.5e-7]) == "  1.00000000E+00 -2.50000000E-07"
    name = S.data_name(2.0, 0.004, "abc", num_particles=16, volume=731.9)
    assert name == "02.000-0016-%06.3f-0.00400-abc" % (16 / 731.9)
    assert S.output_path("OUTPUT", "estimator", name).endswith("ce-estimator-" + name + ".dat")

    # file semantics: new file, restart into it, fresh run over it
    path = os.path.join(tmp_path, "OUTPUT", "ce-estimator-x.dat")
    b = S.Bin(2)
    b.add([1.0, 2.0]); b.add([3.0, 6.0])
    with S.EstimatorFile(path, " " * 15 + "K" + " " * 15 + "V", "id1") as f:
        f.output(b.take(norm=np.array([1.0, 0.5])))
    with S.EstimatorFile(path, "ignored", "id2", restart=True) as f:
        f.output(([4.0, 4.0], 2, 1.0))
    lines = open(path).read().splitlines()
    assert lines == ["# PIMCID: id1", "#" + " " * 14 + "K" + " " * 15 + "V",
                     "  2.00000000E+00  2.00000000E+00", "  2.00000000E+00  2.00000000E+00"]
    with S.EstimatorFile(path, "#  again", "id3", restart=False) as f:
        pass
    assert open(path).read() == "#  again\n"


# ---------------------------------------------------------------------------
# GPU: the generator state and resume
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_plain_rng_state_matches_oracle(pgb, oracle_lib):
    from helpers import make_pair
    n, m, L, lam, tau = 8, 32, 7.5, 6.0596, 0.01
    cfg = wl.seeded_worldlines(n, m, L, lam, tau, 4)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam)
    a.plain_seed(29)
    mt = oracle_lib.MT(29)
    assert np.array_equal(a.rng_state(), mt.save())
    a.plain_run(3, mbar=8, temperature=1 / (m * tau), num_updates=50)
    o.run_steps(mt, 3, mbar=8, temperature=1 / (m * tau), num_updates=50)
    assert np.array_equal(a.rng_state(), mt.save())
    # a state set from outside continues that stream
    mt2 = oracle_lib.MT(77)
    a.set_rng_state(mt2.save())
    o.load(cfg)
    a.load(cfg)
    ra = a.plain_run(2, mbar=8, temperature=1 / (m * tau), num_updates=50, trace_cap=400)
    ro = o.run_steps(mt2, 2, mbar=8, temperature=1 / (m * tau), num_updates=50, trace_cap=400)
    assert np.array_equal(ra["trace"], ro["trace"])


@pytest.mark.gpu
def test_plain_resume_from_state_file(pgb, tmp_path):
    n, m, L, lam, tau = 8, 32, 7.5, 6.0596, 0.01
    T = 1 / (m * tau)
    cfg = wl.seeded_worldlines(n, m, L, lam, tau, 6)
    path = os.path.join(tmp_path, "state")
    a = pgb.Action(L, m, n, tau, lam)
    a.load(cfg)
    a.plain_seed(31)
    a.plain_run(3, mbar=8, temperature=T, num_updates=40)
    S.save_plain_state(a, cfg, path, move_counts=[(5, 10), (6, 12)], estimator_counts=[(0, 0)])
    cont = a.plain_run(4, mbar=8, temperature=T, num_updates=40, trace_cap=1000)
    pos_cont = a.positions()

    b = pgb.Action(L, m, n, tau, lam)
    S.resume_plain_state(b, path, m, L)
    res = b.plain_run(4, mbar=8, temperature=T, num_updates=40, trace_cap=1000)
    # the 16-digit text rounds positions by < 1 ulp: the same moves and
    # decisions follow, energies agree to rounding
    assert np.array_equal(res["trace"], cont["trace"])
    assert np.max(np.abs(res["energies"] - cont["energies"]) /
                  np.maximum(np.abs(cont["energies"]), 1.0)) <= 1e-9
    assert np.max(np.abs(b.positions() - pos_cont)) <= 1e-12


@pytest.mark.gpu
def test_walkers_checkpoint_resume_is_exact(pgb, tmp_path):
    w = wl.workload_walkers(num=12, seed=4, nmax=64)

    def make():
        W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                        seed=11, threads_per_walker=6008)
        W.init()
        return W

    A = make()
    A.run(3, measure=1)
    S.save_walkers(A, str(tmp_path), seed=11)
    A.run(4, measure=1)
    ref = A.all_positions()
    assert np.array_equal(A.sweeps_done(), np.full(12, 7, dtype=np.uint64))

    B = make()
    meta = S.resume_walkers(B, str(tmp_path))
    assert meta["sweeps"] == [3] * 12
    B.run(4, measure=1)
    assert np.array_equal(B.all_positions(), ref)
    assert np.array_equal(B.energy(pgb.PGB_MIXED), A.energy(pgb.PGB_MIXED))
    # each walker's file is a reference state file with identity links
    st = S.parse_state(open(os.path.join(tmp_path, "state2")).read())
    assert st["beads"].shape == (w["m"][1], w["n"][1], 3)
    assert np.array_equal(st["next"][-1, :, 0], np.zeros(w["n"][1], dtype=np.int32))
