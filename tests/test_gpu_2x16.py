"""GPU: the 2x16 two-hole ladder (2.4e9 representatives in the k=(0,0) sector: 64-bit rows).

Size-independent properties at the full size:
* the sizes of all 32 momentum sectors add up to the dimension C(32,2) C(30,15) of the (Nh, Nd) space;
* the fast rows (colex deltas, coset permutations) and the fused step kernels equal the
  reference-faithful orbit walk, FP64.
The mixed-versus-FP64 ground energy of this sector is a measurement (about five minutes), not a test.
"""

import pytest
import scipy.special

pytestmark = pytest.mark.gpu

W = {"tl": 1.0, "tr": 1.0, "jl": 0.5, "jr": 0.5}


def test_2x16_sector_sizes_sum_to_the_space(cuda):
    torch = cuda
    from exactdiag_gb300.engine import DeviceSector

    total = 0
    for kx in range(16):
        for ky in (0, 1):
            sec = DeviceSector(16, 2, 15, kx, ky)
            total += sec.n
            sec.close()
            torch.cuda.empty_cache()
    assert total == scipy.special.comb(32, 2, exact=True) * scipy.special.comb(30, 15, exact=True)


def test_2x16_fast_rows_equal_faithful_orbit_walk(cuda):
    torch = cuda
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(16, 2, 15, 0, 0)
    assert sec.n > 2**31
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(sec.n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    y_walk = sec.hv_mode(x, W, 1)
    scale = float(torch.max(torch.abs(y_walk)).item())
    y = sec.hv_mode(x, W, 0)
    assert float(torch.max(torch.abs(y - y_walk)).item()) < 1e-12 * scale
    y = sec.hv(x, W)  # the fused step kernels: segments of free blocks, 64-bit row offsets
    assert float(torch.max(torch.abs(y - y_walk)).item()) < 1e-12 * scale
    del x, y, y_walk
    sec.close()
    torch.cuda.empty_cache()
