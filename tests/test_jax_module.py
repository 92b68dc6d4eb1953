"""matfun_gb300.jax (custom_vjp over the adjoint FFI handlers): gradient and Hessian-vector product against the
torch.autograd path on the same matrices.  Needs jax with a CUDA backend; skipped where jax is not installed (the
handlers themselves are tested with XLA-style call frames in test_xla_ffi*.py)."""
import numpy as np
import pytest

jax = pytest.importorskip("jax")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fam,kind,alpha", [("smf", "log", None), ("gmf", "pow", 0.3)])
def test_grad_and_hvp_match_torch(fam, kind, alpha):
    import torch

    import matfun_gb300.autograd as ag
    from matfun_gb300 import jax as mj
    from matfun_gb300 import workloads as w
    jax.config.update("jax_enable_x64", True)
    import jax.numpy as jnp
    A = w.c1_gmf_groups(64, seed=3)[:32] if fam == "gmf" else w.c0_smf_spd(32, seed=3, as_voigt=False)
    rng = np.random.default_rng(4)
    W, V = rng.standard_normal((2, len(A), 3, 3))
    f = getattr(mj, fam)
    L = lambda X: (jnp.asarray(W) * f(kind, X, alpha)).sum()
    g = np.asarray(jax.grad(L)(jnp.asarray(A)))
    hv = np.asarray(jax.grad(lambda X: (jax.grad(L)(X) * jnp.asarray(V)).sum())(jnp.asarray(A)))
    r = ag.adjoint(fam, kind, torch.from_numpy(A).cuda(), W=torch.from_numpy(W).cuda(), V=torch.from_numpy(V).cuda(),
                   alpha=alpha, want=("Abar", "HWV"))
    assert np.allclose(g, r["Abar"].cpu().numpy(), rtol=1e-12, atol=0, equal_nan=True)
    assert np.allclose(hv, r["HWV"].cpu().numpy(), rtol=1e-12, atol=0, equal_nan=True)
