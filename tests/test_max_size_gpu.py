"""A batch of more than 2^31 grid points (512^2 x 8200 copies, one FP32 component, 17 GB
of state): every index of the passes, the TMA tile coordinates and the device-side
copies stay in 64-bit range.  The copies are identical, so after two steps each must
equal the single-copy run bit for bit; the comparison runs on the device in chunks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, B = 512, 8200  # 2,149,580,800 points > 2^31


def _problem(gpe, batch, u_one):
    shape = (N, N, batch) if batch > 1 else (N, N)
    u0 = np.zeros(shape, np.complex64, order="F")
    if batch == 1:
        u0[...] = u_one
    return gpe.GrossPitaevskiiProblem((u0,), (64.0, 64.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.05j,
                                      nonlinearity=lambda u, p: 0.2 * np.abs(u[0]) ** 2,
                                      pump=lambda r, p, t: 0.5 * np.exp(-((r[0] - 32) ** 2 + (r[1] - 32) ** 2) / 50.0))


def test_batch_beyond_2_31_points(gpe, lib):
    torch = pytest.importorskip("torch")
    L = gpe._lib
    assert N * N * B > 2 ** 31
    rng = np.random.default_rng(11)
    u_one = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64) * 0.5

    one = gpe.StrangSplittingIterator(_problem(gpe, 1, u_one), (0.0, 1.0), dt=0.01, nsaves=1, device=0)
    one.step(2)
    ref = np.array(one.get_fields()[0])  # Julia order (x, y)
    one.close()

    many = gpe.StrangSplittingIterator(_problem(gpe, B, None), (0.0, 1.0), dt=0.01, nsaves=1, device=0)
    dev = torch.device("cuda:0")
    # [copy][y][x] on the device: the one field repeated (x fastest, as the library stores it)
    f = torch.from_numpy(np.ascontiguousarray(u_one.T)).to(dev)
    big = f.unsqueeze(0).expand(B, N, N).contiguous()
    L.check(lib, many.h, lib.gpe_set_field_dev(many.h, 0, big.data_ptr()))
    many.step(2)
    L.check(lib, many.h, lib.gpe_get_field_dev(many.h, 0, big.data_ptr()))
    torch.cuda.synchronize()
    first = big[0].clone()
    for c0 in range(0, B, 512):
        blk = big[c0:c0 + 512]
        assert bool((blk == first.unsqueeze(0)).all()), c0
    got = first.cpu().numpy().T  # back to (x, y)
    assert np.array_equal(got, ref)
    del big
    many.close()
    torch.cuda.empty_cache()
