"""Tensor-core GEMM and the surrogate MLP against torch FP32 / the FP64
oracle with matching BF16 roundings."""
import numpy as np
import pytest
import torch

import mlp_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import surrogate
    return surrogate


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 512, 320), (384, 64, 128),
                                   (1024, 4096, 512)])
def test_gemm_matches_fp32(S, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    ref = A.float() @ B.float().T
    C = S.gemm_bf16(A, B)
    torch.testing.assert_close(C, ref, rtol=1e-4, atol=1e-3 * float(ref.abs().max()))
    C2, C16 = S.gemm_bf16(A, B, bias=bias, relu=True, out16=True)
    ref2 = torch.relu(ref + bias)
    torch.testing.assert_close(C2, ref2, rtol=1e-4, atol=1e-3 * float(ref.abs().max()))
    torch.testing.assert_close(C16.float(), ref2.to(torch.bfloat16).float(), rtol=1e-2, atol=1e-2)


def test_mlp_gradients_match_oracle(S):
    dims = [72, 256, 256, 128]
    net = S.MLP(dims, max_batch=512, seed=3)
    rng = np.random.Generator(np.random.PCG64(2))
    B = 300  # not a multiple of 128: padded rows must not contribute
    X = rng.normal(size=(B, dims[0])).astype(np.float32)
    T = rng.normal(size=(B, dims[-1])).astype(np.float32)
    p = net.get_params().cpu().numpy()
    loss, g = net.gradients(torch.as_tensor(X), torch.as_tensor(T))
    lo, go = mlp_oracle.loss_and_grads(p, dims, X.astype(np.float64), T.astype(np.float64))
    np.testing.assert_allclose(float(loss), lo, rtol=1e-4)
    g = g.cpu().numpy()
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 2e-2, rel
    Y = net(torch.as_tensor(X)).cpu().numpy()
    Yo, _ = mlp_oracle.forward(p, dims, X.astype(np.float64))
    np.testing.assert_allclose(Y, Yo, rtol=1e-3, atol=1e-3 * np.abs(Yo).max())
    net.close()


def test_mlp_params_roundtrip_and_training(S):
    dims = [16, 128, 128]
    net = S.MLP(dims, max_batch=1024, seed=1)
    p = net.get_params()
    net.set_params(p * 0.5)
    torch.testing.assert_close(net.get_params(), p * 0.5)
    g = torch.Generator(device="cpu").manual_seed(0)
    X = torch.randn(1024, 16, generator=g)
    Wt = torch.randn(16, 128, generator=g)
    T = torch.tanh(X @ Wt)
    hist = net.fit(X.cuda(), T.cuda(), epochs=80, batch=256, lr=3e-3)
    assert hist[-1] < 0.25 * hist[0], hist
    net.close()


def test_checkpoint_resume_is_exact(S, tmp_path):
    """Parameters + Adam moments + step restored into a fresh network: the
    next steps equal those of the network that never stopped."""
    dims = [16, 128, 128]
    g = torch.Generator(device="cpu").manual_seed(3)
    X = torch.randn(512, 16, generator=g).cuda()
    T = torch.tanh(X @ torch.randn(16, 128, generator=g).cuda())
    a = S.MLP(dims, max_batch=512, seed=5)
    for _ in range(5):
        a.train_step(X, T, 2e-3)
    path = str(tmp_path / "mlp.pt")
    a.save(path)
    for _ in range(5):
        a.train_step(X, T, 2e-3)
    b = S.MLP.load(path, max_batch=512)
    assert b.state_dict()["adam_step"] == 5
    for _ in range(5):
        b.train_step(X, T, 2e-3)
    assert torch.equal(a.get_params(), b.get_params())
    sa, sb = a.state_dict(), b.state_dict()
    assert torch.equal(sa["adam_m"], sb["adam_m"]) and torch.equal(sa["adam_v"], sb["adam_v"])
    assert sa["adam_step"] == sb["adam_step"] == 10
    a.close()
    b.close()
