"""A DMFT run restarted from its own restart file: SelfEnergy_w written by dmftgpu_imgfreq_write after three
iterations (dataOut_full, src/ImgTimeFtn.cpp:330-355), read back by dmftgpu_imgfreq_read (read_full,
src/ImgTimeFtn.cpp:673-751) and continued with dmft_main's first TightBinding call (src/dmft_main.cpp:300), against
the same calls on the state that was never written.  The file keeps 8 decimals, so the two agree to that
resolution."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu


def _cm(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(torch.device("cuda:0"))


def _back(t):
    return np.swapaxes(t.cpu().numpy(), -1, -2)


def test_restart_from_written_self_energy(tmp_path):
    import torch
    wl = models.hubbard_2d(kx=32, ky=32, beta=40.0, nfreq=512, ntau=2048, U=2.0)
    uidx, ut = models.gen_Uijkl(2, 2.0, 2.0, 0.0, density_density=True)
    p = dict(ntau=wl.ntau, n_electrons=1.0, U=2.0, Uprime=2.0, J=0.0, mixing=0.5, magnetism=0, dctype=1,
             nominal_charge=1.0, uidx=uidx, ut=ut)
    ctx = lib.Context(0)
    try:
        lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, 2)
        Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=torch.device("cuda:0"))
        Hcm = Hd.transpose(-1, -2).contiguous()
        himp = Hd[:, :2, :2].mean(0)

        def tightbinding(sig):
            """dmft_main's TightBinding call: mu search, G_loc, NumMatrix, Delta (column-major device state)."""
            mu, _ = ctx.GreenFtn_w_adjust_mu(lat, Hd, sig, 0.0, 1.0, 1.0, newton=True)
            gl, _, nm = ctx.GreenFtn_w(lat, Hd, sig, mu, with_gwhf=False)
            we = ctx.Construct_hyb_delta([0, 1], sig, gl, mu, wl.beta, himp)
            t = lambda x: x.transpose(-1, -2).contiguous()
            return mu, [t(sig), t(we), t(nm), t(gl)]

        mu, st = tightbinding(torch.from_numpy(wl.sigma).to(Hd.device))
        for it in range(1, 4):
            mu, _, _ = ctx.DMFT_iteration(lat, Hcm, p, it, *st, mu, newton=True)
        # write SelfEnergy_w (tail slots zero, as the loop's Sigma carries none) and read it back
        se = np.zeros((wl.nfreq + 5, 2, 2), np.complex128)
        se[:wl.nfreq] = _back(st[0])
        path = tmp_path / "Sw_SOLVER.full.dat"
        lib.imgfreq_write(path, se)
        back = lib.imgfreq_read(path, wl.nfreq, 2, wl.beta, wl.beta)
        d = back[:wl.nfreq] - se[:wl.nfreq]   # 8 decimals: each part within half a unit of the last
        assert max(np.abs(d.real).max(), np.abs(d.imag).max()) <= 5e-9 + 1e-15
        mu_r, st_r = tightbinding(torch.from_numpy(np.ascontiguousarray(back[:wl.nfreq])).to(Hd.device))
        mu_c, st_c = tightbinding(st[0].transpose(-1, -2).contiguous())  # the same call on the unwritten state
        assert abs(mu_r - mu_c) < 1e-8
        for a, b in zip(st_r, st_c):
            assert rel_err(_back(a), _back(b)) < 1e-7
        # one more iteration from each (linear mixing: no mixer history): the results agree to the file's resolution
        q = dict(p, pulay_start=100)
        mu_r, _, res_r = ctx.DMFT_iteration(lat, Hcm, q, 1, *st_r, mu_r, newton=True)
        mu_c, _, res_c = ctx.DMFT_iteration(lat, Hcm, q, 1, *st_c, mu_c, newton=True)
        torch.cuda.synchronize()
        assert abs(mu_r - mu_c) < 1e-8 and abs(res_r[0] - res_c[0]) < 1e-7 * max(1.0, abs(res_c[0]))
        for a, b in zip(st_r, st_c):
            assert rel_err(_back(a), _back(b)) < 1e-7
    finally:
        ctx.close()
