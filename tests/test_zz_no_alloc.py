"""The allocation-free diagnostics entry point, mcb_diagnostics_device, against the handle's
mcb_diagnostics.

mcb_diagnostics_device serves callers that cannot call cudaMalloc:
  - host codes that own all device memory through their own pool, sized at start-up;
  - loops that must not risk the device-wide synchronisation cudaFree can imply.
Its only scratch is a file-scope device array that every call shares. So it must give
what mcb_diagnostics gives for the same fields, on one call and on the next, with nothing
left over from the previous call, and the device's free memory must not move across a call.

This file is collected last on purpose. If it fails, a run stopping at the first failure
has already run every other test.
"""
import numpy as np
import pytest

import mcb

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "rho", "ux", "uy", "uz")
# Same fields, same fixed reduction grid and order: these agree exactly.
EXACT = ("umax", "rho_in", "rho_out", "dp", "n_in", "n_out", "vol_half", "phi_min",
         "phi_max", "finite")


def _case(bc, ratio=False):
    nx, ny, nz = 24, 20, 28
    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=bc, tau=0.7, tau_g=1.0, sigma=0.05,
                             width=4.0, sharp_c=0.0)
    if ratio:
        cfg.rho_in, cfg.rho_out = 10.0, 1.0
    phi = mcb.fill_phi_bubbles(nx, ny, nz, bc, 4.0, [(10.8, 10.3, 11.2, 5.0),
                                                     (18.2, 4.4, 21.6, 3.0)])
    u = None
    if bc != mcb.BC_REF:
        rng = np.random.default_rng(5)
        u = tuple((1e-3 * rng.standard_normal(phi.shape)).astype(np.float32) for _ in range(3))
    return cfg, phi, u


def _interior(a, bc):
    return a[1:-1, 1:-1, 1:-1] if bc == mcb.BC_REF else a


@pytest.mark.parametrize("bc,ratio", [(mcb.BC_PERIODIC, False), (mcb.BC_REF, False),
                                      (mcb.BC_WALLS_Z, False), (mcb.BC_PERIODIC, True)])
def test_device_diagnostics_match_the_handle_on_consecutive_calls(bc, ratio):
    # The caller's device arrays; the entry point itself allocates nothing.
    torch = pytest.importorskip("torch")
    cfg, phi, u = _case(bc, ratio)
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *(u if u is not None else (None, None, None)))
        for call in range(2):
            s.step(17)
            want = s.diagnostics()
            host = {k: np.ascontiguousarray(s.get(k)) for k in FIELDS}
            q30 = s.get_phi_q30()
            dev = {k: torch.from_numpy(v).to("cuda") for k, v in host.items()}
            dev_q30 = torch.from_numpy(q30).to("cuda")
            torch.cuda.synchronize()
            args = [dev[k].data_ptr() for k in FIELDS] + [cfg.nx, cfg.ny, cfg.nz, bc]
            free0 = torch.cuda.mem_get_info()[0]
            got = mcb.diagnostics_device(*args, phi_q30=dev_q30.data_ptr())
            free1 = torch.cuda.mem_get_info()[0]
            # with the handle's exact Q2.30 phi the integer mass is the handle's, to the unit
            assert got["mass_q30"] == want["mass_q30"], call
            assert got["mass"] == want["mass"], call
            for k in EXACT:
                assert got[k] == want[k], (call, k, got[k], want[k])
            if ratio:
                # The handle's rho field holds p / cs^2 under a density ratio; this entry
                # point takes it as the density, as documented.
                u2 = sum(host[k].astype(np.float64) ** 2 for k in ("ux", "uy", "uz"))
                ke = 0.5 * float(np.sum(host["rho"].astype(np.float64) * u2))
                assert got["kinetic"] == pytest.approx(ke, rel=1e-9), call
                assert got["kinetic"] != want["kinetic"], call
            else:
                assert got["kinetic"] == want["kinetic"], call
            assert got["update"] == -1
            if call == 1:
                # The first call may load the library's kernels into the context; the next
                # one must leave the device's free memory where it was.
                assert free1 == free0, (free0, free1)
            # Without the Q2.30 array the integer mass comes from phi rounded to Q2.30.
            got_f = mcb.diagnostics_device(*args)
            ints = np.rint(_interior(host["phi"], bc).astype(np.float64) * 2.0 ** 30)
            assert got_f["mass_q30"] == int(ints.astype(np.int64).sum()), call
            assert got_f["mass"] == pytest.approx(want["mass"], rel=1e-6), call
            for k in EXACT:
                assert got_f[k] == want[k], (call, k)


def test_device_diagnostics_reject_oversized_lattices():
    with pytest.raises(mcb.McbError) as e:
        mcb.diagnostics_device(1, 1, 1, 1, 1, 2048, 2048, 1024, mcb.BC_PERIODIC)
    assert e.value.code == mcb.ERR_INVALID
    assert "2^31-1" in str(e.value)
