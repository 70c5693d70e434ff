"""Writes tests/golden/idg_small.npz: a tiny seeded observation and the FP64 oracle's
partition, w-stacked grid, degridded visibilities and dirty image for it.

The reference (C# on .NET Core 3.0) cannot run in this environment, so these vectors
come from the oracle restatement (parity unpinned); they pin the oracle and the GPU
path against regressions.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as entry  # noqa: E402
import oracle  # noqa: E402

synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))


def main():
    wl = synth.scaled_workload("meerkat_3072", n_ant=5, nt=60, nch=4, seed=11)
    wl["obs"]["grid_size"] = 256
    wl["obs"]["cell_arcsec"] = 12.0
    wl["obs"]["n_power_law"] = 6
    wl["obs"]["n_gauss"] = 0
    obs, cd = synth.build(wl)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    layers = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    model_grid = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    degridded, _ = oracle.idg_degrid(cd, subs, model_grid, obs.uvw, obs.frequencies, wstack=True)
    image = oracle.wstack_ifft_float(layers, cd["vis_count"])
    consts = np.array([tuple(cd[k] for k in ("vis_count", "grid_size", "subgrid_size", "kernel_size",
                                            "max_timesteps", "scale_arcsec", "wlayer_count", "wstep"))],
                      dtype=[("vis_count", "<i8"), ("grid_size", "<i4"), ("subgrid_size", "<i4"),
                             ("kernel_size", "<i4"), ("max_timesteps", "<i4"), ("scale_arcsec", "<f4"),
                             ("wlayer_count", "<i4"), ("wstep", "<f8")])[0]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "idg_small.npz")
    np.savez_compressed(out, consts=consts, uvw=obs.uvw, freq=obs.frequencies, vis=obs.vis, subgrids=subs,
                        layers=layers, model_grid=model_grid, degridded=degridded, image=image)
    print(out, len(subs), "subgrids", os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
