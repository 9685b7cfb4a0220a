"""The reference's own GPU kernels (compiled unchanged from its sources into
oracle/_ref/ by oracle/build_ref_gpu.py) launched by oracle/ref_gpu.py with
the reference launchers' grid, checked against the oracle.  They are the
same-GPU baseline the plain kernel is measured against; this pins the
restated launch geometry.  Skipped when the cubins have not been built."""
import numpy as np
import pytest

from helpers import rel_to_max, seeded
from oracle import oracle, ref_gpu

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference cubins not built (oracle/build_ref_gpu.py)")]


@pytest.fixture(scope="module")
def ref():
    return ref_gpu.RefKernels()


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("side", [33, 64])
def test_ccn_shuffle(ref, side):
    left, right = seeded((1, side, side), 81), seeded((1, side, side), 82)
    dl, dr = dev(left), dev(right)
    out = torch.full((1, 2 * side - 1, 2 * side - 1), float("nan"), device="cuda")
    ref.ccn_shuffle(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), side, side, warps=8)
    torch.cuda.synchronize()
    assert rel_to_max(out.cpu().numpy(), oracle.run_mode("one_to_one", left, right)) <= 1e-5


@pytest.mark.parametrize("mats", [1, 2, 8])
def test_multimat_right_work_distribution(ref, mats):
    left, right = seeded((1, 40, 40), 83), seeded((5, 40, 40), 84)
    dl, dr = dev(left), dev(right)
    out = torch.zeros((5, 79, 79), device="cuda")
    ref.multimat_right_work_distribution(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), 40, 40, 5, warps=8, mats=mats,
                                         max_rows=8)
    torch.cuda.synchronize()
    assert rel_to_max(out.cpu().numpy(), oracle.run_mode("one_to_many", left, right)) <= 1e-5


@pytest.mark.parametrize("shifts,mats,rows", [(2, 2, 2), (4, 4, 4), (4, 2, 4)])
def test_one_to_many_multirow_both_multimat_right(ref, shifts, mats, rows):
    left, right = seeded((1, 48, 48), 85), seeded((7, 48, 48), 86)
    dl, dr = dev(left), dev(right)
    out = torch.full((7, 95, 95), float("nan"), device="cuda")
    ref.one_to_many_multirow_both_multimat_right(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), 48, 48, 7, warps=8,
                                                 shifts=shifts, mats=mats, rows=rows)
    torch.cuda.synchronize()
    assert rel_to_max(out.cpu().numpy(), oracle.run_mode("one_to_many", left, right)) <= 1e-5
