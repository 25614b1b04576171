"""kfg_psd: the power spectrogram of tools/psdpng.c (transform_signal,
psdpng.c:116-175) on the GPU, against the same computation in float64
numpy: 16-bit mono and stereo samples, with and without mean removal,
several navg; only whole rows.  The comparison is on the powers
(10^(dB/10) - 1 = mean |X|^2): relative L2 per row <= 2e-5, twice the float
FFT's bound on |X| (a bin near zero -- DC after mean removal -- holds only
rounding noise in any float build, so its dB value is not compared alone)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_psd(x, nfft, navg, stereo, remove_dc):
    x = x.astype(np.int64)
    t = (x[0::2] + x[1::2]) if stereo else x
    nrows = t.size // nfft // navg
    t = t[:nrows * navg * nfft].reshape(nrows * navg, nfft).astype(np.float64)
    if remove_dc:
        t = t - t.mean(axis=1, keepdims=True)
    m = np.abs(np.fft.rfft(t, axis=1)) ** 2
    m = m.reshape(nrows, navg, nfft // 2 + 1).sum(axis=1)
    return 10 * np.log10(m / navg + 1)


@pytest.mark.parametrize("nfft,navg,stereo,remove_dc", [(1024, 4, False, False), (512, 1, True, True),
                                                        (2048, 7, False, True), (480, 3, True, False)])
def test_psd_matches_float64(nfft, navg, stereo, remove_dc):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300 as kf
    rng = np.random.default_rng(nfft + navg)
    n = nfft * navg * 9 + nfft // 3  # a partial row and frame at the end are dropped
    x = rng.integers(-32768, 32768, size=(2 * n if stereo else n,), dtype=np.int64).astype(np.int16)
    got = kf.psd(x, nfft, navg, stereo=stereo, remove_dc=remove_dc)
    ref = reference_psd(x, nfft, navg, stereo, remove_dc)
    assert got.shape == ref.shape == (9, nfft // 2 + 1)
    pg = 10.0 ** (got.astype(np.float64) / 10) - 1
    pr = 10.0 ** (ref / 10) - 1
    err = np.linalg.norm(pg - pr, axis=1) / np.linalg.norm(pr, axis=1)
    assert err.max() <= 2e-5, err.max()
