"""The allocation-free diagnostics entry point, mcb_diagnostics_device, against the handle's
mcb_diagnostics.

mcb_diagnostics_device serves callers that cannot call cudaMalloc:
  - host codes that own all device memory through their own pool, sized at start-up;
  - loops that must not risk the device-wide synchronisation cudaFree can imply.
Its only scratch is a file-scope device array that every call shares. So it must give
what mcb_diagnostics gives for the same fields, on one call and on the next, with nothing
left over from the previous call.

This file is collected last on purpose. If it fails, a run stopping at the first failure
has already run every other test.
"""
import numpy as np
import pytest

import mcb

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "rho", "ux", "uy", "uz")
# Same fields, same fixed reduction grid and order: these agree exactly.
EXACT = ("kinetic", "umax", "rho_in", "rho_out", "dp", "n_in", "n_out", "vol_half",
         "phi_min", "phi_max", "finite")


def _case(bc):
    nx, ny, nz = 24, 20, 28
    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=bc, tau=0.7, tau_g=1.0, sigma=0.05,
                             width=4.0, sharp_c=0.0)
    phi = mcb.fill_phi_bubbles(nx, ny, nz, bc, 4.0, [(10.8, 10.3, 11.2, 5.0),
                                                     (18.2, 4.4, 21.6, 3.0)])
    u = None
    if bc != mcb.BC_REF:
        rng = np.random.default_rng(5)
        u = tuple((1e-3 * rng.standard_normal(phi.shape)).astype(np.float32) for _ in range(3))
    return cfg, phi, u


@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_REF])
def test_device_diagnostics_match_the_handle_on_consecutive_calls(bc):
    # The caller's device arrays; the entry point itself allocates nothing.
    torch = pytest.importorskip("torch")
    cfg, phi, u = _case(bc)
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *(u if u is not None else (None, None, None)))
        for call in range(2):
            s.step(17)
            want = s.diagnostics()
            dev = {k: torch.from_numpy(np.ascontiguousarray(s.get(k))).to("cuda")
                   for k in FIELDS}
            torch.cuda.synchronize()
            got = mcb.diagnostics_device(*(dev[k].data_ptr() for k in FIELDS), cfg.nx, cfg.ny,
                                         cfg.nz, bc)
            for k in EXACT:
                assert got[k] == want[k], (call, k, got[k], want[k])
            # The handle sums the exact Q2.30 phi; from float32 phi the sum agrees to float
            # rounding.
            assert got["mass"] == pytest.approx(want["mass"], rel=1e-6), call
            assert got["update"] == -1


def test_device_diagnostics_reject_oversized_lattices():
    with pytest.raises(mcb.McbError) as e:
        mcb.diagnostics_device(1, 1, 1, 1, 1, 2048, 2048, 1024, mcb.BC_PERIODIC)
    assert e.value.code == mcb.ERR_INVALID
    assert "2^31-1" in str(e.value)
