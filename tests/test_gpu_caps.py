"""The device samplers' iteration caps (the no-trap, no-hang contract).

The reference loops without bound (src/dist/normal.rs:54-67 the ziggurat tail,
the attempt loop of normal.rs:18-43, src/copula/student_t.rs:93-119 the gamma
rejection loop).  The engine's loops stop at a cap, set an error bit, return,
and the host turns the bit into STOCHA_ERR_DEVICE with the cap named in the
message; the context stays usable.  With the product caps no correct draw
comes near them, so stocha_debug_capped_draws lowers one cap to 1 to drive
that path, on 2^20 draws where thousands of attempts (about 1 %), hundreds
of tail draws and gamma rejections need a second iteration.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 20
CASES = [(0, "normal-draw attempt cap reached", 4096), (1, "ziggurat tail iteration cap reached", 4096),
         (2, "normal-draw attempt cap reached", 4096), (3, "ziggurat tail iteration cap reached", 4096),
         (4, "gamma rejection cap reached", 1 << 20)]


@pytest.mark.parametrize("sampler,message,product_cap", CASES)
def test_cap_reports_device_error_and_next_call_is_clean(stocha, oracle, sampler, message, product_cap):
    from stocha_gb300 import _lib

    lib = _lib.load()
    out = np.empty(N)
    rc = lib.stocha_debug_capped_draws(None, sampler, 1, 42, N, _lib.dptr(out))
    assert rc == _lib.STOCHA_ERR_DEVICE
    err = lib.stocha_last_error().decode()
    assert "device check failed" in err and message in err, err
    # the product cap on the same draws: no error, finite values
    _lib.check(lib.stocha_debug_capped_draws(None, sampler, product_cap, 42, N, _lib.dptr(out)))
    assert np.isfinite(out).all()
    # the context is clean for the next call, whose paths are the reference's
    got = stocha.gbm(100.0, 0.05, 0.2, 1.0, 16, 257, seed=42)
    want = oracle.gbm(100.0, 0.05, 0.2, 1.0, 16, 257, seed=42)
    assert np.max(np.abs(got - want) / want) <= 1e-12


def test_cap_argument_checks(stocha):
    from stocha_gb300 import _lib

    lib = _lib.load()
    out = np.empty(4)
    assert lib.stocha_debug_capped_draws(None, 5, 1, 42, 4, _lib.dptr(out)) == _lib.STOCHA_ERR_VALUE
    assert lib.stocha_debug_capped_draws(None, 0, 0, 42, 4, _lib.dptr(out)) == _lib.STOCHA_ERR_VALUE
