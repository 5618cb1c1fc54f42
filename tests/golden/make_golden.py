"""Generate the golden fixtures in this directory from the reference itself.

Run in a container that has the reference checkout (it is not needed anywhere
else; the fixtures are committed):

    python tests/golden/make_golden.py --ref <reference checkout>   (or USCT_REFERENCE=...)

Every case is computed by the reference's Python package ``ringfwi``
(``simulation/ringfwi/fwi.py``) and, for point elements, also by the
reference's own C++ core ``software/core/libuap.hpp`` (compiled by
``oracle/Makefile`` into ``oracle/_ref/``).  The setups mirror the reference's
own tests:

* ring2d_point    -- simulation/tests/test_gradient.py:20-40
* ring2d_aperture -- simulation/tests/test_gradient_aperture.py:161-180
* ring2d_sponge   -- test_gradient.py setup with solver.make_sponge(width=6)
* gn2d            -- simulation/tests/test_gauss_newton.py:234-246
* cyl3d_point     -- simulation/tests/test_gradient_3d.py:94-113
* cyl3d_aperture  -- test_gradient_3d.py setup with build_footprints(rect)
* odd2d / odd3d   -- non-square grids with GridArray elements, one element on
                     the grid border (exercises the lap = 0 border rule)
* parity2d/parity3d -- software/python/test_parity.py:76-90 (the reference's
                     C++-vs-Python parity problems)
* gpu3d           -- software/python/test_gpu.py:139-152 (the reference's
                     FP32-GPU-vs-FP64 parity problem, every third element)
* ring2d_window / cyl3d_window -- the ring2d_point / cyl3d_point problems with
                     per-transmit data windows (fwi.py:247-301 time_weights): a
                     tapered mute after the direct arrival, L2 and GCN
* pwindow2d       -- fwi.p_window_weights (fwi.py:663-699) of the ring2d_point
                     data (and of the parity2d data, 16 transmits)
* footprints      -- geometry.build_footprints (geometry.py:212-278) for rings,
                     cylinders and spherical shells, every aperture shape, and
                     the element indices of SphereArray / HemisphereArray
* tfm2d / tfm3d   -- imaging.tfm (imaging.py:27-74): the reference's point-
                     scatterer dataset of simulation/tests/test_imaging.py:18-38
                     (16-element ring, scattered field only) and a small 3D
                     cylinder analogue; envelope and real-part images
* gn_vs_gd2d      -- simulation/tests/test_gauss_newton.py:54-75: 4 gradient-
                     descent and 4 Gauss-Newton iterations (n_cg 8) of fwi.invert
* pipeline2d      -- simulation/tests/test_pipeline.py:23-59 without the HDF5
                     round trip (no h5py): simulate_dataset, then the "fwi"
                     plugin (fwi_from_dataset) from the flaw-free background
* invert2d        -- fwi.invert (fwi.py:535-660) on the ring2d_point problem
                     with an update mask and bounds as fwi_from_dataset builds
                     them (fwi.py:753-760): 3 steepest-descent iterations (L2),
                     2 with GCN, 2 with the ring2d_window windows, and one
                     truncated Gauss-Newton iteration (fwi.py:434-532)

``--only a,b`` regenerates just the named fixtures.

Each fixture stores the inputs (m, m0, element indices, footprints as CSR,
wavelet, dt, h, nt, src_list, sponge) and the reference outputs (dobs, J, g;
J_gcn, g_gcn for the GCN misfit on point-element cases; Hv for the
Gauss-Newton cases).
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _fp_csr(footprints):
    ptr, cells, w = [0], [], []
    for idxs, ws in footprints:
        for c, wi in zip(idxs, ws):
            cells.append(tuple(int(a) for a in c))
            w.append(float(wi))
        ptr.append(len(cells))
    return np.asarray(ptr, np.int32), np.asarray(cells, np.int32), np.asarray(w)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("USCT_REFERENCE", ""),
                    help="the reference checkout (default: $USCT_REFERENCE)")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(os.path.join(args.ref, "simulation")):
        ap.error("give --ref <reference checkout> or set USCT_REFERENCE")
    only = set(filter(None, args.only.split(",")))

    def want(name):
        return not only or name in only
    sys.path.insert(0, os.path.join(args.ref, "simulation"))
    sys.path.insert(0, REPO)
    from ringfwi import fwi, imaging, phantom, plugins
    from ringfwi.acquire import simulate_dataset
    from ringfwi.geometry import CylinderArray, GridArray, RingArray, build_footprints
    from ringfwi.solver import make_sponge
    from ringfwi.sources import ricker

    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref",
                    f"REF={args.ref}"], check=True)
    import oracle

    def save(name, **kw):
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **kw)
        print(f"wrote {path} ({os.path.getsize(path)} B)")

    def point_case(name, geom, m_true, m0, wav, dt, h, nt, src_list, sponge=None,
                   with_cpp=True):
        if not want(name):
            return
        idx = np.asarray(geom.idx, np.int32)
        dobs = fwi.forward_fmc(m_true, geom, wav, dt, h, nt, sponge, src_list)
        J, g = fwi.misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, sponge, src_list)
        out = dict(m_true=m_true, m0=m0, idx=idx, wavelet=wav, dt=dt, h=h, nt=nt,
                   src_list=np.asarray(src_list, np.int32), dobs=dobs, J=J, g=g,
                   sponge=np.zeros(0) if sponge is None else sponge)
        # the GCN misfit (fwi.py:158-167; libuap.hpp misfit_type=1)
        Jg, gg = fwi.misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, sponge, src_list,
                                         misfit_type="gcn")
        out["J_gcn"] = Jg
        out["g_gcn"] = gg
        if with_cpp:
            out["dobs_cpp"] = oracle.ref_forward_fmc(m_true, geom, wav, dt, h, nt, src_list)
            Jc, gc = oracle.ref_misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, src_list)
            out["J_cpp"] = Jc
            out["g_cpp"] = gc
            Jgc, ggc = oracle.ref_misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, src_list,
                                                      misfit_type="gcn")
            out["J_gcn_cpp"] = Jgc
            out["g_gcn_cpp"] = ggc
            assert np.abs(out["dobs_cpp"] - dobs).max() <= 1e-12 * np.abs(dobs).max()
            assert abs(Jc - J) <= 1e-12 * abs(J)
        save(name, **out)

    def window_case(name, geom, m_true, m0, wav, dt, h, nt, src_list, c_mute, f0, periods):
        """time_weights: W[i][n, j] = 1 up to `periods` periods after the straight-ray
        arrival from transmit i to receiver j at c_mute, then a cosine taper to
        0 over 40 samples (a P-arrival mute as fwi.py:250-253 describes)."""
        if not want(name):
            return
        idx = np.asarray(geom.idx, np.float64)
        t = np.arange(nt) * dt
        W = []
        for s in src_list:
            dist = np.linalg.norm(idx - idx[s], axis=1) * h
            t0 = dist / c_mute + periods / f0
            x = np.clip((t[:, None] - t0[None, :]) / (40 * dt), 0.0, 1.0)
            W.append(0.5 * (1.0 + np.cos(np.pi * x)))
        W = np.asarray(W)
        dobs = fwi.forward_fmc(m_true, geom, wav, dt, h, nt, None, src_list)
        out = dict(m_true=m_true, m0=m0, idx=np.asarray(geom.idx, np.int32), wavelet=wav, dt=dt,
                   h=h, nt=nt, src_list=np.asarray(src_list, np.int32), dobs=dobs,
                   sponge=np.zeros(0), tw=W)
        for mt, sfx in (("l2", ""), ("gcn", "_gcn")):
            J, g = fwi.misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, None, src_list,
                                           misfit_type=mt, time_weights=list(W))
            out["J" + sfx] = J
            out["g" + sfx] = g
            out["Jm" + sfx] = fwi.misfit(m0, geom, wav, dt, h, nt, dobs, None, src_list,
                                         misfit_type=mt, time_weights=list(W))
        save(name, **out)

    # --- 2D ring, point elements (test_gradient.py) ---------------------------
    h = 1.0e-3
    geom = RingArray(n_elements=8, radius_m=0.024, domain_m=0.06, h=h)
    n = geom.n
    dt, nt = 1.2e-7, 350
    wav = ricker(nt, dt, 0.4e6)
    c0 = phantom.coupling_background((n, n), 3000.0, 1480.0, 0.02, h)
    ct = phantom.add_inclusion(c0, (0.5, 0.5), 0.006, 3400.0, h)
    m_true, m0 = phantom.velocity_to_m(ct), phantom.velocity_to_m(c0)
    point_case("ring2d_point", geom, m_true, m0, wav, dt, h, nt, [0, 4])
    window_case("ring2d_window", geom, m_true, m0, wav, dt, h, nt, [0, 4], 1480.0, 0.4e6, 6.0)
    if want("pwindow2d"):
        d_pt = np.load(os.path.join(HERE, "ring2d_point.npz"))["dobs"]
        d_pa = np.load(os.path.join(HERE, "parity2d.npz"))
        save("pwindow2d", W_point=np.asarray(fwi.p_window_weights(d_pt, dt, 0.4e6)),
             dt_point=dt, f0_point=0.4e6,
             W_parity=np.asarray(fwi.p_window_weights(d_pa["dobs"], float(d_pa["dt"]), 0.3e6)),
             dt_parity=float(d_pa["dt"]), f0_parity=0.3e6)

    # --- the reference's Gauss-Newton-vs-descent and pipeline tests ------------
    if want("gn_vs_gd2d"):
        h_g = 1.0e-3
        g_g = RingArray(n_elements=8, radius_m=0.024, domain_m=0.06, h=h_g)
        n_g = g_g.n
        dt_g, nt_g = 1.2e-7, 300
        wav_g = ricker(nt_g, dt_g, 0.4e6)
        c_t = phantom.coupling_background((n_g, n_g), 3000.0, 1480.0, 0.02, h_g)
        c_t = phantom.add_inclusion(c_t, (0.55, 0.5), 0.006, 3350.0, h_g)
        mt_g = phantom.velocity_to_m(c_t)
        m0_g = phantom.velocity_to_m(phantom.coupling_background((n_g, n_g), 3000.0, 1480.0,
                                                                   0.02, h_g))
        sl = [0, 2, 4, 6]
        dobs_g = fwi.forward_fmc(mt_g, g_g, wav_g, dt_g, h_g, nt_g, src_list=sl)
        yy, xx = np.mgrid[0:n_g, 0:n_g].astype(float) * h_g
        cc = (n_g - 1) * h_g / 2
        mask_g = (np.hypot(xx - cc, yy - cc) <= 0.019).astype(float)
        m_gd, hist_gd = fwi.invert(m0_g, g_g, wav_g, dt_g, h_g, nt_g, dobs_g, src_list=sl,
                                   n_iter=4, update_mask=mask_g)
        m_gn, hist_gn = fwi.invert(m0_g, g_g, wav_g, dt_g, h_g, nt_g, dobs_g, src_list=sl,
                                   n_iter=4, update_mask=mask_g, optimizer="gauss-newton",
                                   n_cg=8)
        save("gn_vs_gd2d", m_true=mt_g, m0=m0_g, idx=np.asarray(g_g.idx, np.int32),
             wavelet=wav_g, dt=dt_g, h=h_g, nt=nt_g, src_list=np.asarray(sl, np.int32),
             dobs=dobs_g, sponge=np.zeros(0), mask=mask_g, m_gd=m_gd, hist_gd=np.asarray(hist_gd),
             m_gn=m_gn, hist_gn=np.asarray(hist_gn))
    if want("pipeline2d"):
        h_p = 1.25e-3
        ring_p = RingArray(n_elements=12, radius_m=0.020, domain_m=0.050, h=h_p)
        n_p = ring_p.n
        dt_p, nt_p = 1.2e-7, 360
        wav_p = ricker(nt_p, dt_p, 0.3e6)
        c_bg = phantom.coupling_background((n_p, n_p), 3000.0, 1480.0, 0.016, h_p)
        c_tp = phantom.add_inclusion(c_bg, (0.60, 0.50), 0.005, 2600.0, h_p)
        ds_p = simulate_dataset(c_tp, ring_p, wav_p, dt_p, nominal_speed_m_s=3000.0)
        bounds_p = (phantom.velocity_to_m(3600.0), phantom.velocity_to_m(2500.0))
        res = plugins.run("fwi", ds_p, start_c=c_bg, m_bounds=bounds_p, n_iter=6,
                          step_frac=0.04)
        save("pipeline2d", c_true=c_tp, c_bg=c_bg, idx=np.asarray(ring_p.idx, np.int32),
             element_pos=ds_p.geometry.element_pos, radius_m=ring_p.radius_m, wavelet=wav_p,
             dt=dt_p, h=h_p, nt=nt_p, data=ds_p.data, lo=bounds_p[0], hi=bounds_p[1],
             c_rec=res["c"], history=np.asarray(res["history"]), flaw=np.asarray([0.60, 0.50]))

    # --- the inversion loops (fwi.py:434-660) ----------------------------------
    if want("invert2d"):
        sl = [0, 4]
        dobs = fwi.forward_fmc(m_true, geom, wav, dt, h, nt, None, sl)
        centre = (n - 1) * h / 2.0
        yy, xx = np.mgrid[0:n, 0:n].astype(float) * h
        mask = (np.sqrt((yy - centre) ** 2 + (xx - centre) ** 2)
                <= geom.radius_m * 0.95).astype(float)
        bounds = (1.0 / 3500.0 ** 2, 1.0 / 1400.0 ** 2)
        tw = np.load(os.path.join(HERE, "ring2d_window.npz"))["tw"]
        out = dict(m_true=m_true, m0=m0, idx=np.asarray(geom.idx, np.int32), wavelet=wav, dt=dt,
                   h=h, nt=nt, src_list=np.asarray(sl, np.int32), dobs=dobs, sponge=np.zeros(0),
                   mask=mask, lo=bounds[0], hi=bounds[1], tw=tw)
        runs = {"gd": dict(n_iter=3),
                "gcn": dict(n_iter=2, misfit_type="gcn"),
                "tw": dict(n_iter=2, time_weights=list(tw)),
                "gn": dict(n_iter=1, optimizer="gauss-newton", n_cg=3)}
        for key, kw in runs.items():
            m_rec, hist = fwi.invert(m0, geom, wav, dt, h, nt, dobs, src_list=sl,
                                     update_mask=mask, m_bounds=bounds, step_frac=0.03, **kw)
            out["m_" + key] = m_rec
            out["hist_" + key] = np.asarray(hist)
        save("invert2d", **out)

    # --- element footprints and shell arrays (geometry.py:140-278) -------------
    if want("footprints"):
        from ringfwi.geometry import HemisphereArray, SphereArray
        gs = {"ring": RingArray(n_elements=12, radius_m=0.02, domain_m=0.05, h=1.0e-3),
              "cyl": CylinderArray(n_rings=3, per_ring=10, radius_m=0.012, height_m=0.012,
                                   domain_m=0.032, h=8.0e-4),
              "sphere": SphereArray(20, 0.012, 0.032, 8.0e-4),
              "hemi": HemisphereArray(16, 0.012, 0.032, 8.0e-4)}
        cases = [("flat", 0.004, None), ("rect", 0.005, 0.003), ("disc", 0.005, 0.004),
                 ("point", 0.004, None), ("rect", 0.0005, 0.0005), ("disc", 0.02, 0.02)]
        out = {}
        for gname, gobj in gs.items():
            out[f"{gname}_idx"] = np.asarray(gobj.idx, np.int32)
            for ci, (shp, w, hgt) in enumerate(cases):
                fp = build_footprints(gobj, width_m=w, shape=shp, height_m=hgt)
                p_, c_, w_ = _fp_csr(fp)
                out[f"{gname}_{ci}_ptr"], out[f"{gname}_{ci}_idx"], out[f"{gname}_{ci}_w"] = p_, c_, w_
        save("footprints", **out)

    # --- TFM imaging (imaging.py:27-74) -----------------------------------------
    def tfm_case(name, geom_t, shape, h_t, dt_t, nt_t, f0, centre_frac, radius_scat, npix,
                 half):
        if not want(name):
            return
        wav_t = ricker(nt_t, dt_t, f0)
        c_ref = np.full(shape, 1480.0)
        if len(shape) == 2:
            c_sc = phantom.add_inclusion(c_ref, centre_frac, radius_scat, 3200.0, h_t)
        else:
            c_sc = phantom.add_sphere(c_ref, centre_frac, radius_scat, 3200.0, h_t)
        ds = simulate_dataset(c_sc, geom_t, wav_t, dt_t, nominal_speed_m_s=1480.0)
        ds_ref = simulate_dataset(c_ref, geom_t, wav_t, dt_t, nominal_speed_m_s=1480.0)
        data = ds.data - ds_ref.data
        ds.data = data
        img, axes = imaging.tfm(ds, npix=npix, half_size=half)
        img_re, _ = imaging.tfm(ds, npix=npix, half_size=half, envelope=False)
        domain = (shape[0] - 1) * h_t
        true_pos = np.array([f * domain - domain / 2 for f in centre_frac])
        save(name, data=data, element_pos=ds.geometry.element_pos,
             tx_elements=np.asarray(ds.tx_elements), c=ds.nominal_speed_m_s,
             fs=ds.sample_rate_hz, radius_m=ds.geometry.radius_m, npix=npix, half=half,
             image=img, image_re=img_re, axes=np.stack(axes), true_pos=true_pos)

    ring16 = RingArray(n_elements=16, radius_m=0.020, domain_m=0.050, h=1.0e-3)
    tfm_case("tfm2d", ring16, (ring16.n, ring16.n), 1.0e-3, 1.5e-7, 320, 0.5e6, (0.62, 0.50),
             0.003, 81, 0.018)
    cyl_t = CylinderArray(n_rings=2, per_ring=8, radius_m=0.010, height_m=0.010, domain_m=0.026,
                          h=1.0e-3)
    tfm_case("tfm3d", cyl_t, (cyl_t.n,) * 3, 1.0e-3, 1.5e-7, 220, 0.5e6, (0.5, 0.6, 0.45), 0.002,
             21, 0.008)

    # --- 2D sponge (fwi.py:68-69, 313-314) ------------------------------------
    sp = make_sponge((n, n), width=6)
    point_case("ring2d_sponge", geom, m_true, m0, wav, dt, h, nt, [0, 4], sponge=sp,
               with_cpp=False)

    # --- 2D finite aperture (test_gradient_aperture.py) -----------------------
    if want("ring2d_aperture"):
        fps = build_footprints(geom, width_m=0.003, shape="flat")
        dobs = fwi.forward_fmc(m_true, geom, wav, dt, h, nt, src_list=[0, 4], footprints=fps)
        J, g = fwi.misfit_and_gradient(m0, geom, wav, dt, h, nt, dobs, src_list=[0, 4],
                                       footprints=fps)
        fp_ptr, fp_idx, fp_w = _fp_csr(fps)
        save("ring2d_aperture", m_true=m_true, m0=m0, idx=np.asarray(geom.idx, np.int32),
             wavelet=wav, dt=dt, h=h, nt=nt, src_list=np.asarray([0, 4], np.int32), dobs=dobs,
             J=J, g=g, fp_ptr=fp_ptr, fp_idx=fp_idx, fp_w=fp_w, sponge=np.zeros(0))

    # --- 2D Gauss-Newton Hv (test_gauss_newton.py) ----------------------------
    if want("gn2d"):
        nt_gn = 300
        wav_gn = ricker(nt_gn, dt, 0.4e6)
        rng = np.random.default_rng(2)
        v = rng.standard_normal((n, n))
        v[:5] = v[-5:] = v[:, :5] = v[:, -5:] = 0.0
        v *= float(np.mean(m0))
        Hv = fwi.gn_hessian_vector(m0, geom, wav_gn, dt, h, nt_gn, v, src_list=[0, 4])
        save("gn2d", m0=m0, idx=np.asarray(geom.idx, np.int32), wavelet=wav_gn, dt=dt, h=h,
             nt=nt_gn, src_list=np.asarray([0, 4], np.int32), v=v, Hv=Hv, sponge=np.zeros(0))

    # --- 3D cylinder, point elements (test_gradient_3d.py) ---------------------
    h3 = 1.5e-3
    cyl = CylinderArray(n_rings=2, per_ring=6, radius_m=0.010, height_m=0.012,
                        domain_m=0.03, h=h3)
    n3 = cyl.n
    dt3, nt3 = 1.5e-7, 140
    wav3 = ricker(nt3, dt3, 0.35e6)
    c3 = phantom.cylinder_background((n3, n3, n3), 3000.0, 1480.0, 0.008, h3)
    ct3 = phantom.add_sphere(c3, (0.5, 0.5, 0.5), 0.004, 2700.0, h3)
    point_case("cyl3d_point", cyl, phantom.velocity_to_m(ct3), phantom.velocity_to_m(c3),
               wav3, dt3, h3, nt3, [0, 6])
    window_case("cyl3d_window", cyl, phantom.velocity_to_m(ct3), phantom.velocity_to_m(c3),
                wav3, dt3, h3, nt3, [0, 6], 1480.0, 0.35e6, 1.5)

    # --- 3D finite aperture (rect footprints) ---------------------------------
    if want("cyl3d_aperture"):
        fps3 = build_footprints(cyl, width_m=0.004, shape="rect", height_m=0.003)
        mt3, m03 = phantom.velocity_to_m(ct3), phantom.velocity_to_m(c3)
        dobs3 = fwi.forward_fmc(mt3, cyl, wav3, dt3, h3, nt3, src_list=[0, 6], footprints=fps3)
        J3, g3 = fwi.misfit_and_gradient(m03, cyl, wav3, dt3, h3, nt3, dobs3, src_list=[0, 6],
                                         footprints=fps3)
        fp_ptr, fp_idx, fp_w = _fp_csr(fps3)
        save("cyl3d_aperture", m_true=mt3, m0=m03, idx=np.asarray(cyl.idx, np.int32),
             wavelet=wav3, dt=dt3, h=h3, nt=nt3, src_list=np.asarray([0, 6], np.int32),
             dobs=dobs3, J=J3, g=g3, fp_ptr=fp_ptr, fp_idx=fp_idx, fp_w=fp_w,
             sponge=np.zeros(0))

    # --- odd, non-square grids with an element on the border -------------------
    rs = np.random.default_rng(7)
    shp2 = (37, 53)
    idx2 = [(int(rs.integers(3, shp2[0] - 3)), int(rs.integers(3, shp2[1] - 3)))
            for _ in range(5)] + [(0, 20), (36, 52)]
    g2 = GridArray(idx=idx2, n=shp2[0], h=1.0e-3, radius_m=0.015, domain_m=0.036)
    c2 = 1500.0 + 60.0 * rs.standard_normal(shp2)
    point_case("odd2d", g2, phantom.velocity_to_m(c2), phantom.velocity_to_m(np.full(shp2, 1500.0)),
               ricker(200, 1.5e-7, 0.35e6), 1.5e-7, 1.0e-3, 200, [0, 3, 5, 6])

    # --- the reference's own parity problems (test_parity.py, test_gpu.py) ----
    ring16 = RingArray(n_elements=16, radius_m=0.024, domain_m=0.060, h=6e-4)
    n16 = ring16.n
    cp2 = phantom.coupling_background((n16, n16), 3000.0, 1480.0, 0.020, 6e-4)
    cp2 = phantom.add_inclusion(cp2, (0.58, 0.46), 0.006, 2650.0, 6e-4)
    point_case("parity2d", ring16, phantom.velocity_to_m(cp2),
               phantom.velocity_to_m(np.full((n16, n16), np.mean(cp2))),
               ricker(500, 7e-8, 0.3e6), 7e-8, 6e-4, 500, list(range(16)))
    cylp = CylinderArray(n_rings=3, per_ring=12, radius_m=0.015, height_m=0.014,
                         domain_m=0.036, h=1.25e-3)
    npc = cylp.n
    cp3 = phantom.cylinder_background((npc, npc, npc), 3000.0, 1480.0, 0.012, 1.25e-3)
    cp3 = phantom.add_sphere(cp3, (0.56, 0.5, 0.5), 0.005, 2650.0, 1.25e-3)
    point_case("parity3d", cylp, phantom.velocity_to_m(cp3),
               phantom.velocity_to_m(np.full((npc, npc, npc), np.mean(cp3))),
               ricker(250, 1.2e-7, 0.3e6), 1.2e-7, 1.25e-3, 250, list(range(0, 36, 4)))
    cg3 = phantom.cylinder_background((npc, npc, npc), 3000.0, 1480.0, 0.015 * 0.8, 1.25e-3)
    cg3 = phantom.add_sphere(cg3, (0.56, 0.5, 0.5), 0.005, 2650.0, 1.25e-3)
    point_case("gpu3d", cylp, phantom.velocity_to_m(cg3),
               phantom.velocity_to_m(np.full((npc, npc, npc), 3000.0)),
               ricker(250, 1.2e-7, 0.3e6), 1.2e-7, 1.25e-3, 250, list(range(0, 36, 3)))

    shp3 = (13, 17, 21)
    idx3 = [(int(rs.integers(2, shp3[0] - 2)), int(rs.integers(2, shp3[1] - 2)),
             int(rs.integers(2, shp3[2] - 2))) for _ in range(5)] + [(0, 8, 10), (6, 16, 3)]
    g3d = GridArray(idx=idx3, n=shp3[0], h=1.0e-3, radius_m=0.008, domain_m=0.02)
    c3d = 1500.0 + 60.0 * rs.standard_normal(shp3)
    point_case("odd3d", g3d, phantom.velocity_to_m(c3d),
               phantom.velocity_to_m(np.full(shp3, 1500.0)), ricker(120, 1.5e-7, 0.35e6),
               1.5e-7, 1.0e-3, 120, [0, 2, 5, 6])


if __name__ == "__main__":
    main()
