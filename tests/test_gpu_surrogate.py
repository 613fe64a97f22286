"""The displacement surrogate on the GPU against a plain PyTorch fp32
reference of the same operations.

Layers (tensor-core convolutions and the CUDA-core weight gradient) take
BF16 tensors; the reference runs in fp32 on the same BF16-rounded values, so
the only differences are FP32 summation order and the BF16 rounding of the
outputs: a BF16 output within 1e-2 of the largest reference value, FP32
outputs and gradients within 1e-4 relative.  The whole network is compared
with a reference that rounds every stored activation to BF16 as the network
does (relative L2 within 2e-2).  Training must lower the loss; the learned
PCG start must leave the converged answer unchanged (compliance within 1e-8
of the previous-displacement start) and must fall back to the history start
when the network returns non-finite values."""
import ctypes as C

import numpy as np
import pytest

from sparlab_gb300 import _lib
from sparlab_gb300 import problems as P

pytestmark = pytest.mark.gpu


def torch_mod():
    import torch
    return torch


def bf16_tensor(a, dev):
    torch = torch_mod()
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev).to(torch.bfloat16).contiguous()


def to_ncdhw(t):
    """[z][y][x][c] -> [1][c][z][y][x] (fp32)"""
    return t.float().permute(3, 0, 1, 2).unsqueeze(0)


def from_ncdhw(t):
    return t[0].permute(1, 2, 3, 0)


def torch_weight(w):
    """[27][cout][cin] (t = 9 (dz+1) + 3 (dy+1) + (dx+1)) -> [cout][cin][3][3][3]"""
    cout, cin = w.shape[1], w.shape[2]
    return w.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2).contiguous()


def conv(nx, ny, nz, ins, cseg, w, n, bias=None, relu=0, flip=0, outs=None, out_c=None, out_pitch=None,
         out_f32=None):
    lib = _lib.load()
    nseg = len(ins)
    in_ptrs = (C.c_void_p * 2)(*[t.data_ptr() for t in ins], *([0] * (2 - nseg)))
    cs = (C.c_int32 * 2)(*cseg, *([0] * (2 - nseg)))
    nout = len(outs)
    out_ptrs = (C.c_void_p * 2)(*[t.data_ptr() for t in outs], *([0] * (2 - nout)))
    oc = (C.c_int32 * 2)(*out_c, *([0] * (2 - nout)))
    op = (C.c_int32 * 2)(*out_pitch, *([0] * (2 - nout)))
    of = (C.c_int32 * 2)(*out_f32, *([0] * (2 - nout)))
    code = lib.simp_conv3d_bf16(C.c_int32(nx), C.c_int32(ny), C.c_int32(nz), C.c_int32(nseg), in_ptrs, cs,
                                C.c_void_p(w.data_ptr()), C.c_int32(n),
                                C.c_void_p(bias.data_ptr() if bias is not None else 0), C.c_int32(relu),
                                C.c_int32(flip), C.c_int32(nout), out_ptrs, oc, op, of)
    if code:
        _lib.raise_for(code, lib.simp_surrogate_last_error().decode())


@pytest.mark.parametrize("cseg,cout,grid,relu", [
    ((16,), 16, (37, 7, 5), 0),      # ragged tiles in x and y
    ((32,), 64, (32, 8, 3), 1),
    ((64,), 64, (45, 6, 4), 1),
    ((64,), 128, (33, 5, 3), 0),
    ((64, 32), 32, (40, 9, 4), 1),   # concatenated input
    ((32, 16), 16, (31, 4, 3), 1),
    ((64, 64), 64, (20, 4, 2), 1),
])
def test_conv_forward_matches_torch(cseg, cout, grid, relu):
    torch = torch_mod()
    import torch.nn.functional as F
    dev = torch.device("cuda", 0)
    nx, ny, nz = grid
    rng = np.random.default_rng(sum(cseg) * 7 + cout)
    xs = [bf16_tensor(rng.standard_normal((nz, ny, nx, c)), dev) for c in cseg]
    cin = sum(cseg)
    w = bf16_tensor(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin), dev)
    bias = torch.from_numpy(rng.standard_normal(cout).astype(np.float32)).to(dev)
    out = torch.full((nz, ny, nx, cout), float("nan"), dtype=torch.bfloat16, device=dev)
    conv(nx, ny, nz, xs, cseg, w, cout, bias=bias, relu=relu, outs=[out], out_c=[cout], out_pitch=[cout],
         out_f32=[0])
    torch.cuda.synchronize()
    x = torch.cat([to_ncdhw(t) for t in xs], dim=1)
    ref = F.conv3d(x, torch_weight(w.float()), bias=bias, padding=1)
    if relu:
        ref = torch.relu(ref)
    ref = from_ncdhw(ref)
    err = (out.float() - ref).abs().max().item()
    assert err <= 1e-2 * ref.abs().max().item(), err


def test_conv_head_fp32_output_matches_torch():
    torch = torch_mod()
    import torch.nn.functional as F
    dev = torch.device("cuda", 0)
    nx, ny, nz = 35, 6, 3
    rng = np.random.default_rng(5)
    x = bf16_tensor(rng.standard_normal((nz, ny, nx, 16)), dev)
    w = np.zeros((27, 16, 16), np.float32)
    w[:, :3, :] = rng.standard_normal((27, 3, 16)) / 20.0
    wt = bf16_tensor(w, dev)
    out = torch.full((nz, ny, nx, 3), float("nan"), dtype=torch.float32, device=dev)
    conv(nx, ny, nz, [x], (16,), wt, 16, outs=[out], out_c=[3], out_pitch=[3], out_f32=[1])
    torch.cuda.synchronize()
    ref = from_ncdhw(F.conv3d(to_ncdhw(x), torch_weight(wt.float()), padding=1))[..., :3]
    err = (out - ref).abs().max().item()
    assert err <= 1e-4 * ref.abs().max().item(), err


@pytest.mark.parametrize("cseg,cout,grid", [((16,), 16, (37, 7, 5)), ((64,), 32, (33, 5, 4)),
                                             ((64, 32), 32, (40, 9, 3)), ((64, 64), 64, (21, 6, 3))])
def test_conv_data_gradient_matches_torch(cseg, cout, grid):
    """flip = 1 with the transposed weights: the gradient of the convolution
    with respect to its (concatenated) input."""
    torch = torch_mod()
    import torch.nn.functional as F
    dev = torch.device("cuda", 0)
    nx, ny, nz = grid
    cin = sum(cseg)
    rng = np.random.default_rng(cin + cout)
    w = bf16_tensor(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin), dev)
    g = bf16_tensor(rng.standard_normal((nz, ny, nx, cout)), dev)
    wt = w.permute(0, 2, 1).contiguous()    # [27][cin][cout]
    outs = [torch.full((nz, ny, nx, c), float("nan"), dtype=torch.bfloat16, device=dev) for c in cseg]
    conv(nx, ny, nz, [g], (cout,), wt, cin, flip=1, outs=outs, out_c=list(cseg), out_pitch=list(cseg),
         out_f32=[0] * len(cseg))
    torch.cuda.synchronize()
    x = torch.zeros((1, cin, nz, ny, nx), device=dev, requires_grad=True)
    y = F.conv3d(x, torch_weight(w.float()), padding=1)
    y.backward(to_ncdhw(g))
    ref = from_ncdhw(x.grad)
    got = torch.cat([o.float() for o in outs], dim=3)
    err = (got - ref).abs().max().item()
    assert err <= 1e-2 * ref.abs().max().item(), err


@pytest.mark.parametrize("cseg,cout,grid", [((16,), 16, (37, 7, 5)), ((32,), 64, (30, 9, 4)),
                                             ((64, 32), 32, (25, 6, 3))])
def test_weight_gradient_matches_torch(cseg, cout, grid):
    torch = torch_mod()
    import torch.nn.functional as F
    dev = torch.device("cuda", 0)
    lib = _lib.load()
    nx, ny, nz = grid
    cin = sum(cseg)
    rng = np.random.default_rng(3 * cin + cout)
    xs = [bf16_tensor(rng.standard_normal((nz, ny, nx, c)), dev) for c in cseg]
    dy = bf16_tensor(rng.standard_normal((nz, ny, nx, cout)), dev)
    gw = torch.zeros((27, cout, cin), dtype=torch.float32, device=dev)
    gb = torch.zeros(cout, dtype=torch.float32, device=dev)
    in_ptrs = (C.c_void_p * 2)(*[t.data_ptr() for t in xs], *([0] * (2 - len(xs))))
    cs = (C.c_int32 * 2)(*cseg, *([0] * (2 - len(cseg))))
    code = lib.simp_conv3d_wgrad(C.c_int32(nx), C.c_int32(ny), C.c_int32(nz), C.c_int32(len(cseg)), in_ptrs, cs,
                                 C.c_void_p(dy.data_ptr()), C.c_int32(cout), C.c_int32(cout),
                                 C.c_void_p(gw.data_ptr()), C.c_void_p(gb.data_ptr()))
    if code:
        _lib.raise_for(code, lib.simp_surrogate_last_error().decode())
    x = torch.cat([to_ncdhw(t) for t in xs], dim=1)
    wref = torch.zeros((cout, cin, 3, 3, 3), device=dev, requires_grad=True)
    bref = torch.zeros(cout, device=dev, requires_grad=True)
    F.conv3d(x, wref, bias=bref, padding=1).backward(to_ncdhw(dy))
    ref = wref.grad.permute(2, 3, 4, 0, 1).reshape(27, cout, cin)
    assert (gw - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()
    assert (gb - bref.grad).abs().max().item() <= 1e-4 * bref.grad.abs().max().item()


def reference_network(layers, x, dev):
    """The surrogate's forward pass in fp32 PyTorch, rounding every stored
    activation to BF16 as the network stores it."""
    torch = torch_mod()
    import torch.nn.functional as F
    k1 = torch.tensor([0.5, 1.0, 0.5], device=dev)
    k3 = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :])

    def rb(t):
        return t.to(torch.bfloat16).float()

    def P(t):
        c = t.shape[1]
        return rb(F.conv_transpose3d(t, k3.expand(c, 1, 3, 3, 3), stride=2, padding=1, groups=c))

    def R(t):
        c = t.shape[1]
        return rb(F.conv3d(t, k3.expand(c, 1, 3, 3, 3) / 8.0, stride=2, padding=1, groups=c))

    def cv(i, t, relu=True):
        w, b = layers[i]
        wt = torch.from_numpy(w).to(dev).to(torch.bfloat16).float()
        y = F.conv3d(t, torch_weight(wt), bias=torch.from_numpy(b).to(dev), padding=1)
        return rb(torch.relu(y)) if relu else y

    s0 = cv(1, cv(0, x))
    s1 = cv(3, cv(2, R(s0)))
    s2 = cv(5, cv(4, R(s1)))
    b3 = cv(7, cv(6, R(s2)))
    d2 = cv(8, torch.cat([P(b3), s2], 1))
    d1 = cv(9, torch.cat([P(d2), s1], 1))
    d0 = cv(10, torch.cat([P(d1), s0], 1))
    return cv(11, d0, relu=False)


def test_network_forward_matches_torch():
    torch = torch_mod()
    from sparlab_gb300.surrogate import Surrogate
    dev = torch.device("cuda", 0)
    sur = Surrogate(seed=3)
    p = sur.get_params()
    rng = np.random.default_rng(9)
    p[:] += rng.standard_normal(p.size).astype(np.float32) * 0.01   # non-zero biases too
    sur.set_params(p)
    nx, ny, nz = 33, 17, 9      # odd: every level lines up with stride-2 transfers
    x = np.zeros((nz, ny, nx, 16), np.float32)
    x[..., :4] = rng.uniform(-1.0, 1.0, (nz, ny, nx, 4))
    xin = bf16_tensor(x, dev)
    out = torch.zeros((nz, ny, nx, 3), dtype=torch.float32, device=dev)
    sur.forward(nx, ny, nz, xin.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    ref = from_ncdhw(reference_network(sur.layer_params(p), to_ncdhw(xin), dev))
    rel = (torch.linalg.vector_norm(out - ref) / torch.linalg.vector_norm(ref)).item()
    assert rel <= 2e-2, rel


def test_network_gradient_matches_torch_autograd():
    """The composed backward pass (data gradients through the decoder, the
    skip connections and the grid transfers; weight and bias gradients) against
    torch autograd on the reference network, layer by layer.  The reference
    rounds activations and their gradients to BF16 where the network stores
    them (tensor hooks); what remains is summation order and the skip
    connections' gradient sums, which the network rounds per contribution
    (the first layer, behind every other, differs most: about 3 %)."""
    torch = torch_mod()
    import torch.nn.functional as F
    from sparlab_gb300.surrogate import LAYER_NAMES, Surrogate
    dev = torch.device("cuda", 0)
    sur = Surrogate(seed=4)
    p = sur.get_params()
    rng = np.random.default_rng(12)
    p[:] += rng.standard_normal(p.size).astype(np.float32) * 0.01
    sur.set_params(p)
    nx, ny, nz = 49, 25, 17     # level 3: 7 x 4 x 3 nodes
    x = np.zeros((nz, ny, nx, 16), np.float32)
    x[..., :4] = rng.uniform(-1.0, 1.0, (nz, ny, nx, 4))
    xin = bf16_tensor(x, dev)
    tgt = bf16_tensor(rng.uniform(-1.0, 1.0, (nz, ny, nx, 3)), dev)
    mask_np = np.full((nz, ny, nx), 7, np.uint8)
    mask_np[:, :, 0] = 0                     # a clamped face
    mask = torch.from_numpy(mask_np).to(dev)
    count = int(3 * (mask_np > 0).sum())
    loss, g = sur.loss_gradient(nx, ny, nz, xin.data_ptr(), tgt.data_ptr(), mask.data_ptr(), count)
    params = [(torch.from_numpy(w.copy()).to(dev).requires_grad_(True),
               torch.from_numpy(b.copy()).to(dev).requires_grad_(True)) for w, b in sur.layer_params(p)]
    k1 = torch.tensor([0.5, 1.0, 0.5], device=dev)
    k3 = k1[:, None, None] * k1[None, :, None] * k1[None, None, :]

    def rb(t):
        """BF16 storage of an activation and of its gradient"""
        t = t.to(torch.bfloat16).float()
        if t.requires_grad:
            t.register_hook(lambda gr: gr.to(torch.bfloat16).float())
        return t

    def P(t):
        c = t.shape[1]
        return rb(F.conv_transpose3d(t, k3.expand(c, 1, 3, 3, 3), stride=2, padding=1, groups=c))

    def R(t):
        c = t.shape[1]
        return rb(F.conv3d(t, k3.expand(c, 1, 3, 3, 3) / 8.0, stride=2, padding=1, groups=c))

    def cv(i, t, relu=True):
        w, b = params[i]
        y = F.conv3d(t, torch_weight(w.to(torch.bfloat16).float()), bias=b, padding=1)
        return rb(torch.relu(y)) if relu else y

    xt = to_ncdhw(xin)
    s0 = cv(1, cv(0, xt))
    s1 = cv(3, cv(2, R(s0)))
    s2 = cv(5, cv(4, R(s1)))
    b3 = cv(7, cv(6, R(s2)))
    d2 = cv(8, torch.cat([P(b3), s2], 1))
    d1 = cv(9, torch.cat([P(d2), s1], 1))
    d0 = cv(10, torch.cat([P(d1), s0], 1))
    head = cv(11, d0, relu=False)
    head.register_hook(lambda gr: gr.to(torch.bfloat16).float())
    out = from_ncdhw(head)
    m = torch.stack([(mask >> k) & 1 for k in range(3)], dim=-1).float()
    ref_loss = (((out - tgt.float()) ** 2) * m).sum() / count
    ref_loss.backward()
    assert abs(loss / ref_loss.item() - 1) < 1e-2
    off = 0
    for name, (w, b) in zip(LAYER_NAMES, params):
        gw = g[off: off + w.numel()].reshape(w.shape)
        off += w.numel()
        gb = g[off: off + b.numel()]
        off += b.numel()
        rw = w.grad.cpu().numpy()
        rel = np.linalg.norm(gw - rw) / np.linalg.norm(rw)
        assert rel < 5e-2, (name, rel)
        rbias = b.grad.cpu().numpy()
        assert np.linalg.norm(gb - rbias) / np.linalg.norm(rbias) < 5e-2, name


def _small_specs():
    specs = []
    for s in range(3):
        spec = P.hex8_cantilever(24, 12, 12, 0.2 + 0.05 * s, f"sg{s}")
        spec.rtol = 1e-8
        specs.append(spec)
    return specs


def test_training_lowers_the_loss_and_learned_start_keeps_the_answer():
    from sparlab_gb300.surrogate import Surrogate, generate_samples
    from sparlab_gb300.topopt import GpuSimpProblem
    sur = Surrogate(seed=5)
    generate_samples(sur, _small_specs(), iterations=5)
    assert sur.num_samples == 15
    losses = sur.train(epochs=40, learning_rate=1e-3, batch=1, seed=1)
    # the first epoch starts from a near-zero prediction (its loss is about
    # the mean squared target); training must get well below it
    assert all(np.isfinite(losses)) and losses[-1] < 0.3 * losses[0], losses
    runs = {}
    for warm in (1, 3):
        spec = P.hex8_cantilever(24, 12, 12, 0.25, "sg_run")
        spec.rtol = 1e-10
        spec.warm_start = warm
        prob = GpuSimpProblem(spec, precision="mixed")
        if warm == 3:
            prob.set_surrogate(sur)
        runs[warm] = [prob.iterate() for _ in range(4)]
        if warm == 3:
            assert prob.learned_seconds() > 0.0
        prob.close()
    for a, b in zip(runs[1], runs[3]):
        assert abs(a.compliance / b.compliance - 1) < 1e-8


def test_learned_start_falls_back_on_a_non_finite_network():
    """A network that returns NaN adds nothing to the start: warm start 3 then
    computes exactly warm start 2 (the history's energy-optimal start), and
    its first solve starts from zero."""
    from sparlab_gb300.surrogate import Surrogate
    from sparlab_gb300.topopt import GpuSimpProblem
    sur = Surrogate(seed=5)
    sur.set_params(np.full(sur.num_params, np.nan, np.float32))
    recs = {}
    for warm in (2, 3):
        spec = P.hex8_cantilever(20, 10, 10, 0.25, "sg_nan")
        spec.rtol = 1e-9
        spec.warm_start = warm
        prob = GpuSimpProblem(spec, precision="fp64")
        if warm == 3:
            prob.set_surrogate(sur)
        recs[warm] = [prob.iterate() for _ in range(3)]
        prob.close()
    assert [r.compliance for r in recs[2]] == [r.compliance for r in recs[3]]
    assert [r.linear_iterations for r in recs[2]] == [r.linear_iterations for r in recs[3]]
