"""Host side of the served path (no GPU): device sizing of structures,
arrival process and the served workload family."""
import numpy as np

from giraffe_gb300 import configs, gpu, serve


def test_device_bytes_of_a_batch_is_at_most_the_sum_of_its_parts():
    a, b = configs.pipe_chain(40, 0.4, 0.03, [1e5, 0, 0]), configs.pipe_chain(300, 0.35, 0.02, [0, 1e5, 0])
    na, nb, nab = gpu.device_bytes([a]), gpu.device_bytes([b]), gpu.device_bytes([a, b])
    assert 0 < na < nb
    assert max(na, nb) < nab <= na + nb
    # the band (35 doubles per free DOF) dominates: at least that much
    assert nb >= 35 * 8 * b.n_free


def test_device_bytes_rejects_an_invalid_model():
    s = configs.pipe_chain(10, 0.4, 0.03, [1e5, 0, 0])
    s.beams[3] = (s.beams[3][0], s.beams[3][1], 10 ** 6, *s.beams[3][3:])
    try:
        gpu.device_bytes([s])
    except RuntimeError:
        return
    raise AssertionError("an out-of-range node was accepted")


def test_poisson_arrivals():
    t = serve.poisson_arrivals(20000, 200.0, seed=3)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 200.0) < 200.0 * 0.03
    assert np.array_equal(t, serve.poisson_arrivals(20000, 200.0, seed=3))


def test_served_chains_span_the_dof_range():
    s = configs.served_chains(400, seed=1)
    dof = np.array([x.n_free for x in s])
    assert dof.min() >= 900 and dof.max() <= 50100
    assert np.median(dof) > 3000 and np.median(dof) < 15000


def test_served_mixed_stream_shares_and_sizes():
    s = configs.served_mixed(120, seed=4, plate_dof=(10000, 40000))
    plates = [x for x in s if x.shells]
    chains = [x for x in s if x.beams]
    assert len(plates) + len(chains) == 120
    assert 0.18 < len(plates) / 120 < 0.42
    pd = np.array([x.n_free for x in plates])
    assert pd.min() > 7000 and pd.max() < 46000
    assert [x.n_free for x in s][:20] == [x.n_free for x in configs.served_mixed(20, seed=4, plate_dof=(10000, 40000))]
