"""Gaussian-process external potential against the oracle's restatement of
the reference CPU path (GaussianProcessPotential::GP with MaternKernel::K,
GPHeBenzenePotential::V)."""
import os

import numpy as np
import pytest

from pimc_gb300 import worldlines as wl


def test_param_and_training_files(tmp_path):
    from pimc_gb300 import gp
    w = wl.workload_gp(points=37, seed=3)
    tf = os.path.join(tmp_path, "train.dat")
    w["training"].astype("<f8").tofile(tf)
    pf = os.path.join(tmp_path, "gp.ini")
    with open(pf, "w") as f:
        f.write("kernel.type = matern\nkernel.maternNu = 1.5\nkernel.ell = 0.5\nkernel.ell = 1\n"
                "kernel.ell = 2 # comment\nkernel.numTrainingPoints = 37\n"
                f"kernel.trainingFileName = {tf}\n")
    g = gp.read_gp_params(pf)
    assert g["kernel.ell"] == ["0.5", "1", "2"] and g["kernel.maternNu"] == "1.5"
    assert np.array_equal(gp.read_training(tf, 37), w["training"])
    with pytest.raises(ValueError):
        gp.read_training(tf, 38)


def test_oracle_gp_at_known_point(oracle_lib):
    """One training point, r on it: K = 1, V = mean_d + std_d (mu + sigma2 w)."""
    p = dict(matern_nu=2.5, ell=[1, 1, 1], norm_offset=[0, 0, 0], norm_scale=[1, 1, 1],
             standard_mean=2.0, standard_std=3.0, mean=0.5, sigma2=4.0, side=[10, 10, 10])
    v = oracle_lib.gp_eval([[0.1, 0.2, 0.3, 0.25]], [[0.1, 0.2, 0.3]], **p)
    assert v[0] == 2.0 + 3.0 * (0.5 + 4.0 * 0.25)
    # periodic image: a point one box side away sees the same training point
    v2 = oracle_lib.gp_eval([[0.1, 0.2, 0.3, 0.25]], [[10.1, 0.2, -9.7]], **p)
    assert abs(v2[0] - v[0]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("nu", [0.5, 1.5, 2.5])
def test_gp_fp64_matches_oracle(pgb, oracle_lib, nu):
    from pimc_gb300.gp import GaussianProcess
    w = wl.workload_gp(points=700, num_ptcl=16, num_slices=40, seed=1, matern_nu=nu)
    g = GaussianProcess(w["training"], **w["params"])
    got = g(w["pos"])
    want = oracle_lib.gp_eval(w["training"], w["pos"], **w["params"])
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= 1e-12


@pytest.mark.gpu
def test_gp_boundary_conditions_follow_the_cpu_kernel(pgb, oracle_lib):
    """A side short enough that separations wrap: the device applies putInBC
    as MaternKernel::K does; without periodicity the values differ."""
    from pimc_gb300.gp import GaussianProcess
    w = wl.workload_gp(points=300, num_ptcl=8, num_slices=25, seed=2)
    for periodic in ([1, 1, 1], [0, 0, 1], [0, 0, 0]):
        p = dict(w["params"], side=[1.3, 1.7, 1.1], periodic=periodic)
        got = GaussianProcess(w["training"], **p)(w["pos"])
        want = oracle_lib.gp_eval(w["training"], w["pos"], **p)
        assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= 1e-12
        if periodic == [1, 1, 1]:
            wrapped = got
    assert np.max(np.abs(wrapped - got)) > 1e-3


@pytest.mark.gpu
def test_gp_mixed_error_bound(pgb, oracle_lib):
    from pimc_gb300 import PGB_MIXED
    from pimc_gb300.gp import GaussianProcess
    w = wl.workload_gp(points=4096, num_ptcl=32, num_slices=32, seed=4)
    got = GaussianProcess(w["training"], precision=PGB_MIXED, **w["params"])(w["pos"])
    want = oracle_lib.gp_eval(w["training"], w["pos"], **w["params"])
    # FP32 kernel values: error bounded by ~1e-6 of std sigma2 sum |w|
    p = w["params"]
    scale = p["standard_std"] * p["sigma2"] * np.abs(w["training"][:, 3]).sum()
    assert np.max(np.abs(got - want)) <= 1e-6 * scale


@pytest.mark.gpu
def test_gp_benzene_matches_oracle(pgb, oracle_lib):
    from pimc_gb300.gp import GaussianProcess
    w = wl.workload_gp(points=500, num_ptcl=40, num_slices=25, seed=6)
    pos = w["pos"].copy()
    pos[:50, 2] *= 0.1          # some points inside the hard core
    pos[50:60] *= 3.0           # and some far out, in the long-range switch
    g = GaussianProcess(w["training"], **w["params"])
    got = g.benzene(pos)
    want = oracle_lib.gp_eval(w["training"], pos, benzene=True, **w["params"])
    assert np.sum(want == 10000.0) > 0
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= 1e-11


@pytest.mark.gpu
def test_gp_argument_errors(pgb):
    from pimc_gb300.gp import GaussianProcess
    w = wl.workload_gp(points=10, seed=1)
    with pytest.raises(pgb.PgbError):
        GaussianProcess(w["training"], **dict(w["params"], matern_nu=2.0))
    g = GaussianProcess(w["training"], **w["params"])
    assert len(g(np.zeros((0, 3)))) == 0
