"""The CUDA path (through the C ABI, from the reference's file formats)
against golden vectors produced by the reference itself."""
import pytest

import colo
from golden_check import CASES, assert_matches_golden, load, paths

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


@pytest.mark.parametrize("mode", [colo.MODE_PLAIN, colo.MODE_BATCHED])
@pytest.mark.parametrize("case", CASES)
def test_cuda_path_reproduces_reference_golden(ctx, case, mode):
    g = load(case)
    csv, par = paths(case)
    ds = colo.Dataset.from_csv(ctx, str(csv))
    assert ds.names() == g["features"]
    p = colo.read_params(str(par))
    p.mode = mode
    p.keep_tables = 1
    res = ctx.mine(ds, p)
    assert_matches_golden(res, g)
