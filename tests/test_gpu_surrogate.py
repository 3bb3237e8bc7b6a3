"""Learned surrogate force on the GPU: the tensor-core dense layer against a
torch FP32 matmul of the same bf16 operands (up to 50,001 rows, 391 tiles
of 128), the whole CUDA forward against
the torch restatement of the network (bf16 rounding emulated), and the
surrogate HMC step's exact-Hamiltonian bookkeeping.

Tolerances: dense layer within 2 bf16 ulps of the FP32 reference (outputs are
rounded to bf16, accumulation order differs); network forces within 2e-2
relative (norm-wise; bf16 activations through three rounds)."""
import ctypes

import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C(built):
    from trimem_gb300 import capi
    return capi


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("rows", [128, 1000, 4097, 50001])
def test_dense_layer_matches_fp32_matmul(C, rows):
    import torch

    g = torch.Generator(device="cuda").manual_seed(rows)
    h = torch.randn(rows, 64, device="cuda", generator=g).to(torch.bfloat16)
    m = torch.randn(rows, 64, device="cuda", generator=g).to(torch.bfloat16)
    W = (0.1 * torch.randn(64, 128, device="cuda", generator=g)).to(torch.bfloat16)
    b = 0.1 * torch.randn(64, device="cuda", generator=g)
    out = torch.full((rows, 64), float("nan"), device="cuda").to(torch.bfloat16)
    C.check(C.lib().tm_dense_silu_bf16(_p(h), _p(m), _p(W), _p(b), _p(out), rows, None))
    torch.cuda.synchronize()
    x = torch.cat([h, m], 1).float()
    ref = h.float() + torch.nn.functional.silu(x @ W.float().t() + b)
    err = (out.float() - ref).abs()
    assert torch.isfinite(out.float()).all()
    assert (err <= 2 * 2.0 ** -8 * ref.abs().clamp(min=1.0)).all(), float(err.max())


def _random_blob(p, f, seed):
    import torch

    from trimem_gb300 import surrogate as S

    torch.manual_seed(seed)
    net = S.make_net()
    lbar, abar = S.mesh_scales(p, f)
    with torch.no_grad():
        net.scales.copy_(torch.tensor([lbar, abar, 50.0]))
        net.wo.normal_(0, 0.3)
        net.wn.normal_(0, 0.3)
    return net, S.to_blob(net)


def test_surrogate_forward_matches_torch_network(C):
    import torch

    from trimem_gb300 import surrogate as S

    p, f = meshgen.jittered_icosphere(4, seed=3)
    prm = dict(workload_params(p, f, kappa_b=20.0), cont_lambda=0.0)
    mesh = C.Mesh(p, f)
    en = C.Energy(mesh, C.params(**prm))
    net, blob = _random_blob(p, f, 1)
    sg = C.Surrogate(mesh, blob)
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    inp = S.Inputs(sg, en, mesh, x, 16)
    assert inp.nbr.shape[0] == 6  # icosphere valences 5 and 6
    g = torch.empty_like(x)
    C.check(C.lib().tm_surrogate_gradient_device(sg.h, en.h, mesh.h, _p(x), _p(g), None))
    torch.cuda.synchronize()
    F_cuda = (inp.gloc - g).float()
    net = net.cuda()
    with torch.no_grad():
        F_ref = net(inp.u, inp.nrm, inp.nbr, inp.ef, inp.dirs, bf16=True)
    rel = float(torch.linalg.norm(F_cuda - F_ref) / torch.linalg.norm(F_ref))
    assert rel < 2e-2, rel
    # the exact local part: g_local equals the FP32-stencil gradient with the
    # bending and repulsion weights set to zero
    prm0 = dict(prm, kappa_b=0.0, kappa_r=0.0)
    m0 = C.Mesh(p, f)
    e0 = C.Energy(m0, C.params(**prm0))
    _, g0 = e0.gradient(m0, with_energy=True)
    gl = inp.gloc.cpu().numpy()
    assert np.linalg.norm(gl - g0) <= 1e-5 * np.linalg.norm(g0)


def test_surrogate_hmc_step_uses_the_exact_hamiltonian(C):
    import torch

    p, f = meshgen.jittered_icosphere(3, seed=4)
    prm = dict(workload_params(p, f, kappa_b=20.0), cont_lambda=0.0)
    mesh = C.Mesh(p, f)
    en = C.Energy(mesh, C.params(**prm))
    _, blob = _random_blob(p, f, 2)
    sg = C.Surrogate(mesh, blob)
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    out4 = (ctypes.c_double * 4)()
    props = (ctypes.c_double * 6)()
    # no leapfrog steps: H(end) == H(start), always accepted, exact energy
    C.check(C.lib().tm_surrogate_hmc_step_device(sg.h, en.h, mesh.h, _p(x), 1.0, 1e-6, 0, 1.0, 3, 0, 0.5, out4,
                                                 props, None))
    assert out4[0] == 1.0 and out4[1] == out4[2]
    assert out4[3] == pytest.approx(en.energy(mesh), rel=1e-12)
    np.testing.assert_allclose(props[:], en.properties(mesh), rtol=1e-12)
    # with steps: the returned energy is exact at the returned state
    acc = 0
    for k in range(4):
        C.check(C.lib().tm_surrogate_hmc_step_device(sg.h, en.h, mesh.h, _p(x), 1.0, 1e-7, 3, 1.0, 3, k + 1, 0.0,
                                                     out4, props, None))
        acc += int(out4[0])
    mesh.points()[:] = x.cpu().numpy()
    assert out4[3] == pytest.approx(en.energy(mesh), rel=1e-12)
    assert np.isfinite(out4[1]) and np.isfinite(out4[2])


@pytest.fixture(scope="module")
def eq065(C):
    """The learned-surrogate chains' state: the 163,842-vertex benchmark
    membrane at the reduced-volume target 0.65 (one of the training volumes)
    in equilibrium at T 1 (the committed chain state; else equilibrated_state,
    about a minute)."""
    from trimem_gb300 import surrogate as S
    from trimem_gb300.mc.device import equilibrated_state
    from trimem_gb300.mc.equilibrate import load_state
    from trimem_gb300.workloads import workload_params as wp

    if not __import__("os").path.exists(S.WEIGHTS_L7):
        pytest.skip("no trained weights")
    p, f = meshgen.jittered_icosphere(7, seed=0)
    prm = wp(p, f, kappa_b=20.0, vfrac=0.65)
    st = load_state(prm, len(p))
    return st if st is not None else equilibrated_state(p, f, prm, seed=4242)


def _handles(C, st):
    import torch

    mesh = C.Mesh(st["x"], st["faces"])
    if st["topo"] is not None:
        mesh.set_topology(st["topo"])
    en = C.Energy(mesh, C.params(**st["prm"]))
    en.set_initial_props(st["initial"])
    x = torch.tensor(st["x"], dtype=torch.float64, device="cuda").contiguous()
    C.check(C.lib().tm_energy_update_repulsion_device(en.h, mesh.h, _p(x), None))
    return mesh, en, x


def test_trained_network_lowers_the_force_error(C, eq065):
    """On the equilibrated state, the surrogate gradient g_local - F_nn is far
    closer to the exact gradient than g_local alone (the leapfrog force with
    no learned part)."""
    import torch

    from trimem_gb300 import surrogate as S

    mesh, en, x = _handles(C, eq065)
    L = C.lib()
    g_exact = torch.empty_like(x)
    C.check(L.tm_energy_eval_device(en.h, mesh.h, _p(x), _p(g_exact), None, None))
    sg = C.Surrogate(mesh, np.load(S.WEIGHTS_L7))
    g_sur = torch.empty_like(x)
    C.check(L.tm_surrogate_gradient_device(sg.h, en.h, mesh.h, _p(x), _p(g_sur), None))
    inp = S.Inputs(sg, en, mesh, x, 16)
    torch.cuda.synchronize()
    ref = float(torch.linalg.norm(g_exact))
    err_net = float(torch.linalg.norm(g_sur - g_exact)) / ref
    err_none = float(torch.linalg.norm(inp.gloc - g_exact)) / ref
    print(f"relative gradient error: surrogate {err_net:.3e}, without the network {err_none:.3e}")
    assert err_none > 0.005, err_none  # bending and repulsion: a sizeable part of the force here
    assert err_net < 0.25 * err_none, (err_net, err_none)


def test_trained_network_conserves_the_hamiltonian(C, eq065):
    """What the learned force gains inside the sampler: from the equilibrated
    state, surrogate-driven HMC moves (20 velocity-Verlet steps at dt 1e-6,
    the exact FP64 Hamiltonian at both ends) with the trained network end
    with far smaller Hamiltonian errors |H1 - H0|, and so far higher
    acceptance, than the same moves with the network's output set to zero
    (the leapfrog on g_local alone).  The exact-force moves are printed
    beside them: plain HMC remains the better sampler on this energy."""
    from trimem_gb300 import surrogate as S

    mesh, en, x = _handles(C, eq065)
    L = C.lib()
    blob = np.load(S.WEIGHTS_L7)
    zero = blob.copy()
    zero[-(2 * S.H + 2):] = 0.0  # w_o, b_o, w_n, b_n: F = 0
    out = {}
    for name, w in (("trained", blob), ("zero", zero), ("exact", None)):
        sg = C.Surrogate(mesh, w) if w is not None else None
        dh = []
        for k in range(8):
            xc = x.clone()
            o4 = (ctypes.c_double * 4)()
            pr = (ctypes.c_double * 6)()
            if sg is None:
                C.check(L.tm_hmc_step_device(en.h, mesh.h, _p(xc), 1.0, 1e-6, 20, 1.0, 77, k, 0.5, o4, pr, None))
            else:
                C.check(L.tm_surrogate_hmc_step_device(sg.h, en.h, mesh.h, _p(xc), 1.0, 1e-6, 20, 1.0, 77, k, 0.5,
                                                       o4, pr, None))
            dh.append(o4[2] - o4[1])
        out[name] = np.array(dh)
    med = {k: float(np.median(np.abs(v))) for k, v in out.items()}
    acc = {k: float(np.mean(np.minimum(1.0, np.exp(-v)))) for k, v in out.items()}
    print(f"median |H1 - H0|: {med}; mean acceptance probability: {acc}")
    assert np.isfinite(out["trained"]).all()
    assert med["trained"] < 0.25 * med["zero"], med
    assert acc["trained"] > acc["zero"] + 0.2, acc
