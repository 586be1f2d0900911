"""The torch.autograd.Function wrapper (mmo_gb300.torch_ops) on the GPU.

float32 pose tensors of shape [4096, 14] (the energy+gradient workload:
48-atom ligand with 8 torsions, 6,000-atom pocket); energies and gradients
through autograd must equal the C ABI's, and match the FP64 oracle."""
import numpy as np
import pytest

from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return synth.pose_batch(n_poses=4096, seed=1)


def test_autograd_energy_and_gradient(oracle, scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300.torch_ops import uff_score

    from contract import assert_ref, ref_batch

    sc = scorer_factory(system.pocket, system.ligand)
    dev = torch.device("cuda", 0)
    dofs = torch.from_numpy(system.poses).to(dev).requires_grad_(True)
    assert tuple(dofs.shape) == (4096, 14) and dofs.dtype == torch.float32
    E = uff_score(dofs, sc)
    w = torch.linspace(0.5, 1.5, len(E), device=dev, dtype=torch.float64)
    (w * E).sum().backward()
    E_abi, G_abi, _ = sc.score_poses(system.poses, grad=True)
    assert np.array_equal(E.detach().cpu().numpy(), E_abi)
    g = dofs.grad.cpu().numpy()
    assert np.allclose(g, w.cpu().numpy().astype(np.float32)[:, None] * G_abi, rtol=1e-6,
                       atol=0)
    # every pose of the [4096, 14] batch against the FP64 oracle
    assert_ref(E_abi, G_abi, ref_batch(oracle, system, system.poses, grad=True))


def test_autograd_without_grad(scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300.torch_ops import uff_score

    sc = scorer_factory(system.pocket, system.ligand)
    dofs = torch.from_numpy(system.poses[:64]).cuda()
    E = uff_score(dofs, sc)
    assert not E.requires_grad
    E_abi, _, _ = sc.score_poses(system.poses[:64])
    assert np.array_equal(E.cpu().numpy(), E_abi)
