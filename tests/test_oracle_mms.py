"""The oracle on the Poisson manufactured solution of the reference's Poisson
application (tests/mms_cases.py): the L_inf error of the cell values falls
at second order in the cell size, as the scheme's order says."""
import numpy as np

import oracle_lib
from mms_cases import oracle_solve

ORDER_RATIO = (3.5, 4.5)  # error(h) / error(h/2) of a second-order scheme


def test_poisson_mms_converges_at_second_order():
    errs = []
    for n in (16, 32):
        x, ex, _ = oracle_solve(oracle_lib, n)
        errs.append(np.abs(x - ex).max())
    ratio = errs[0] / errs[1]
    assert ORDER_RATIO[0] < ratio < ORDER_RATIO[1], (errs, ratio)
    assert errs[1] < 1e-2
