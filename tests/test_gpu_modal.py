"""Modal analysis on the CUDA path (gf_modal / gf_structure_modal: the
static tangent and the modal mass mounted on the device, K factored once by
the wide-band LU, subspace iteration on K^-1 M) against the reference's
matrices and the oracle.  Stated tolerances: eigenvalues 1e-7 relative to
the golden ones (a dense solver's error on the smallest eigenvalue of these
stiff problems is about eps |lambda_max| / |lambda|); each mode's residual
|K x - lambda M x| / (lambda |M x|) below 1e-5 on the reference's own K and
M (subspace iteration converges the modes at the square root of the rate of
the eigenvalues, which stop at 1e-12); modes M-orthonormal to 1e-9."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from giraffe_gb300.model import Structure
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ref_modal_cantilever.npz", "ref_modal_plate.npz", "ref_modal_riser.npz"])
def test_modal_matches_reference_matrices(gpu_ctx, golden, name):
    g = golden(name)
    s = Structure.from_inp(str(g["deck"]))
    n_modes = len(g["eig"])
    eig, V, its = gpu_ctx.modal(s, n_modes, tol=1e-12)
    assert np.abs(eig - g["eig"]).max() <= 1e-7 * np.abs(g["eig"]).max()
    K, M = g["K"], g["M"]
    for k in range(n_modes):
        x = V[k]
        r = K @ x - eig[k] * (M @ x)
        assert np.linalg.norm(r) <= 1e-5 * eig[k] * np.linalg.norm(M @ x), k
    assert np.allclose(V @ M @ V.T, np.eye(n_modes), atol=1e-9)
    assert 2 <= its <= 300


def test_modal_of_a_structure_after_load_steps_matches_the_oracle(gpu_ctx):
    """gf_structure_modal on a device-resident structure: at the start it is
    gf_modal's result; the modes of a pipe riser under internal pressure
    (its load stiffness symmetric at the undeformed state) match the
    oracle's."""
    s = configs.pipe_riser(12, steps=10)
    ds = gpu.DeviceStructure(gpu_ctx, s)
    eig, V, _ = ds.modal(s.solution.start_time + 5 * s.solution.time_step, 6, tol=1e-12)
    ds.close()
    s2 = configs.pipe_riser(12, steps=10)
    s2.solution.start_time = 5 * s.solution.time_step
    w, _ = oracle.modal(s2, 6)
    assert np.abs(eig - w).max() <= 1e-7 * np.abs(w).max()


def test_nonsymmetric_tangent_is_refused(gpu_ctx):
    """A tip moment's pseudo-moment load stiffness makes K_AA nonsymmetric:
    the symmetric subspace iteration refuses it."""
    s = configs.cantilever_rollup()
    s.solution.start_time = 0.5  # the tip moment is on
    with pytest.raises(RuntimeError, match="not symmetric"):
        gpu_ctx.modal(s, 4)
