"""The adjoint pass pt_adjoint (needs a GB300) in the adjoint-spin setting:
B0 = 1 uT along z plus eight harmonic terms with l <= 2, E = 1e6 V/m along z,
specular walls, spins starting along x.

Criteria:
* the adjoint's own forward pass equals pt_integrate bit for bit;
* the gradients do not depend on the checkpoint interval K (the chunks are
  recomputed with the forward's arithmetic): K = 256, 1024, 4096 agree to
  1e-13 relative;
* adjoint vs central finite differences (h = 1e-3 |G|) of the GPU forward
  pass, for the mean phase, the mean S_x and the mean S_y: within 1e-5 of
  the largest gradient component of each observable;
* the same against finite differences of the oracle's forward pass (the
  oracle evaluates the harmonic field in its own arithmetic order, so its
  trajectories differ by rounding);
* the polarisation |<S>| within 1e-3 of its largest component: its
  gradient, (<S>.d<S>)/|<S>|, is a cancelling combination of the S_x and S_y
  gradients about 1e-6 of their size, so their 1e-8-relative differences to
  finite differences show up magnified.  Those differences are the same for
  the GPU and the oracle: finite differences also see the Bloch step-size
  controller (tolerance 1e-12) answer the perturbed field, which the
  pathwise adjoint, with its accepted step sequence frozen, does not;
* the torch.autograd.Function of the gradient harness gives the adjoint's
  gradient;
* a diffuse wall makes the call fail with PT_ERR_UNSUPPORTED."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu

N, T = 64, 0.1


def setup(n=N, simtime=T):
    from pentrack_gb300 import workloads
    terms = workloads.harmonic_terms_l2()
    sc, params, parts = workloads.adjoint_spin(n=n, simtime=simtime, terms=terms)
    params.mode = A.MODE_PLAIN
    params.field_precision = A.PREC_FP64
    return terms, sc, params, parts


@pytest.fixture(scope="module")
def case(built):
    from pentrack_gb300 import Engine, spin_gradients as SG
    terms, sc, params, parts = setup()
    e = Engine(sc)
    fwd, _ = e.integrate(params, parts)
    grads = {}
    for name in ("phase", "sx", "sy", "polarisation"):
        grads[name] = {}
        for K in (256, 1024, 4096):
            g, out, st = e.adjoint(params, parts, 1, SG.observable_cotangents(fwd, name), checkpoint_interval=K)
            grads[name][K] = g
    return terms, sc, params, parts, e, fwd, out, grads


def test_adjoint_forward_equals_integrate(case):
    terms, sc, params, parts, e, fwd, out, grads = case
    for k in ("t", "y", "spin", "stop_id", "n_hit", "n_accepted"):
        assert np.array_equal(getattr(fwd, k), getattr(out, k)), k


def test_adjoint_independent_of_checkpoint_interval(case):
    grads = case[-1]
    for name, gk in grads.items():
        ref = gk[1024]
        scale = np.abs(ref).max()
        for K, g in gk.items():
            assert np.max(np.abs(g - ref)) <= 1e-13 * scale, (name, K)


def _fd(terms, params, parts, integrate):
    from pentrack_gb300 import spin_gradients as SG, workloads
    return SG.fd_gradients(lambda c: workloads.adjoint_spin_scene(terms=c), terms, params, parts, integrate=integrate, rel_step=1e-3)


TOL = {"phase": 1e-5, "sx": 1e-5, "sy": 1e-5, "polarisation": 1e-3}


def _compare(grads, fd):
    for name, tol in TOL.items():
        g = grads[name][1024]
        scale = np.abs(fd[name]).max()
        assert scale > 0, name
        np.testing.assert_array_less(np.abs(g - fd[name]), tol * scale, err_msg=name)


def test_adjoint_matches_gpu_finite_differences(case):
    from pentrack_gb300 import Engine
    terms, sc, params, parts, e, fwd, out, grads = case
    base, fd = _fd(terms, params, parts, lambda s, p, ps: Engine(s).integrate(p, ps)[0])
    _compare(grads, fd)


def test_adjoint_matches_oracle_finite_differences(case, oracle_mod):
    terms, sc, params, parts, e, fwd, out, grads = case
    base, fd = _fd(terms, params, parts, lambda s, p, ps: oracle_mod.Oracle(s).integrate(p, ps)[0])
    _compare(grads, fd)


def test_autograd_harness_uses_the_adjoint(case):
    torch = pytest.importorskip("torch")
    from pentrack_gb300 import spin_gradients as SG, workloads
    terms, sc, params, parts, e, fwd, out, grads = case
    f = SG.make_spin_tracking(lambda c: workloads.adjoint_spin_scene(terms=c), terms, params, parts)
    g = torch.tensor([t[2] for t in terms], dtype=torch.float64, requires_grad=True)
    spins = f.apply(g)
    loss = spins[4].mean()  # the mean phase
    (dg,) = torch.autograd.grad(loss, g)
    ref = grads["phase"][1024]
    assert np.max(np.abs(dg.numpy() - ref)) <= 1e-12 * np.abs(ref).max()


def test_adjoint_rejects_diffuse_walls(built):
    from pentrack_gb300 import Engine, spin_gradients as SG, workloads
    from pentrack_gb300.engine import EngineError
    terms, sc, params, parts = setup(n=32, simtime=0.5)
    sc.materials[1] = workloads.storage_vacuum(0.5, 0.0)[1:]
    e = Engine(sc)
    fwd, _ = e.integrate(params, parts)
    with pytest.raises(EngineError) as ex:
        e.adjoint(params, parts, 1, SG.observable_cotangents(fwd, "phase"))
    assert ex.value.status == A.PT_ERR_UNSUPPORTED
