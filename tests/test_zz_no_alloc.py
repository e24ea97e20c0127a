"""The allocation-free spectrum binner (axs_powerspec_noalloc) against the
allocating entry point (axs_powerspec) and the oracle on the same field.

axs_powerspec_noalloc is for callers that own every byte of device memory
and cannot have this library call cudaMalloc/cudaFree: they bring the R2C
spectrum and the output buffers, the library brings only the kernels and a
static scratch array. Here torch plays that caller: it owns the buffers and
runs the FFT; the call goes through the C ABI.

This file sorts last so that a run stopping at the first failure has run
every other test before it. It also passes on its own in a fresh process
(the first call does the per-device set-up itself).
"""
import numpy as np
import pytest

from gpu_util import orc, params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,N,precision,tol", [(3, 32, 64, 1e-11), (2, 64, 64, 1e-11), (3, 48, 32, 1e-5)])
def test_noalloc_binner_matches_powerspec_twice(axs, oracle, nd, N, precision, tol):
    torch = pytest.importorskip("torch")
    p = params(axs, nd, N, precision)
    rdt = torch.float64 if precision == 64 else torch.float32
    with axs.Lattice(p) as L:
        L.init_thermal(13)
        L.evolve(4)
        fields = L.download()
        wants = [L.powerspec(axs.PHI2), L.powerspec(axs.PHI1)]
    nb = N // 2
    pk = torch.empty(nb, dtype=torch.float64, device="cuda")
    ks = torch.empty(nb, dtype=torch.float64, device="cuda")
    cnt = torch.empty(nb, dtype=torch.int32, device="cuda")
    for field, want in zip((fields[1], fields[0]), wants):   # two calls in a row, different inputs
        x = torch.from_numpy(np.ascontiguousarray(field)).to(device="cuda", dtype=rdt)
        spec = torch.fft.rfftn(x).contiguous()                  # cuFFT R2C layout [N][N][N/2+1]
        pk.fill_(-1.0)
        ks.fill_(-1.0)
        cnt.fill_(-1)
        stream = torch.cuda.current_stream().cuda_stream
        axs.powerspec_noalloc(spec.data_ptr(), nd, N, precision, p.space_step, pk.data_ptr(), ks.data_ptr(),
                              cnt.data_ptr(), stream)
        torch.cuda.synchronize()
        pk_h, ks_h, cnt_h = pk.cpu().numpy(), ks.cpu().numpy(), cnt.cpu().numpy()
        pk_w, ks_w, cnt_w = want
        assert np.array_equal(cnt_h, cnt_w)
        ok = cnt_w > 0
        assert np.abs(pk_h[ok] - pk_w[ok]).max() <= tol * np.abs(pk_w[ok]).max()
        assert np.abs(ks_h[ok] - ks_w[ok]).max() <= tol * np.abs(ks_w[ok]).max()
        assert np.all(np.isnan(pk_h[~ok])) and np.all(np.isnan(pk_w[~ok]))
        # and directly against the oracle's output_powerspec of the same field
        pk_o, ks_o, cnt_o = oracle.powerspec(orc(p), field)
        assert np.array_equal(cnt_h, cnt_o)
        assert np.abs(pk_h[ok] - pk_o[ok]).max() <= tol * np.abs(pk_o[ok]).max()
        assert np.abs(ks_h[ok] - ks_o[ok]).max() <= tol * np.abs(ks_o[ok]).max()


def test_noalloc_binner_rejects_sizes_beyond_its_scratch(axs):
    with pytest.raises(axs.AxsError) as e:
        axs.powerspec_noalloc(1 << 20, 3, 4096, 32, 0.5, 1 << 20, 1 << 20, 1 << 20)
    assert e.value.code == axs.ERR_ARG
    assert "at most 1024" in str(e.value)
