"""Generate the golden fixtures in tests/golden/ from the reference's own kernels.

Each fixture is a small seeded scene run stage by stage through the reference's
kernel sources compiled as host C++ (oracle/_ref/libsphref.so, built by
oracle/ref/build_ref.sh from the reference checkout). The npz file stores the
parameters, the initial records and the output of every stage; tests replay
the same stages through the oracle (bit-identical) and the CUDA library
(within tolerance) on machines where the reference checkout does not exist.

Run from the repository root, with SPH_REFERENCE_ROOT naming the reference
checkout:  SPH_REFERENCE_ROOT=<checkout> python tests/golden/make_golden.py
"""
import json
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "sph-multiphase_gb300"), os.path.join(REPO, "tests")]

from oracle import oracle as O  # noqa: E402
from sphmp import abi, scenes  # noqa: E402

from golden_stages import SIDE_STAGES, STAGES, prepare_multiphase, state_arrays  # noqa: E402


def fixtures():
    """(name, scene, multiphase seed) of every fixture."""
    out = []
    out.append(("tait3_block", scenes.small_block(seed=21, n=(9, 7, 8), nphase=3, eos=abi.EOS_TAIT,
                                                  velocity_scale=0.4, walls=False, box=(0.2, 0.2, 0.2))))
    out.append(("tait2_walls", scenes.small_block(seed=22, n=(6, 5, 6), nphase=2, eos=abi.EOS_TAIT,
                                                    velocity_scale=0.2, box=(0.08, 0.08, 0.08))))
    sc = scenes.small_block(seed=23, n=(8, 8, 8), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3, walls=False,
                            simscale=0.5, h=0.01, d=0.01, box=(0.2, 0.2, 0.2))
    out.append(("simscale_half", sc))
    # out-of-grid particles: outermost cell layer, outside, non-finite
    sc = scenes.small_block(seed=24, n=(8, 7, 6), nphase=1, eos=abi.EOS_TAIT, velocity_scale=0.2, walls=False,
                            box=(0.2, 0.2, 0.2))
    p = sc.params
    lo = np.array(p.gridmin, np.float32)
    cell = np.float32(p.cellsize / p.simscale)
    sc.disp["pos"][3] = lo + 0.5 * cell
    sc.disp["pos"][11] = lo - 1.0
    sc.disp["pos"][17] = (np.nan, 0.1, 0.1)
    sc.disp["pos"][29, 1] = np.float32(p.gridmin[1] + p.gridsize[1]) - np.float32(0.25) * cell
    out.append(("out_of_grid", sc))
    sc = scenes.small_block(seed=25, n=(7, 7, 7), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3, walls=False,
                            box=(0.2, 0.2, 0.2))
    sc.params.surface_tension = 1
    sc.params.surfaceTensionK = 1.0
    sc.params.surfaceTensionFluidC = 0.05
    out.append(("surface_tension", sc))
    # liquid phases only (no gas next to liquid), so that the project-U force, which
    # squares drift velocities, stays finite; boundary factors other than 1
    sc = scenes.small_block(seed=26, n=(6, 6, 5), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.4,
                            dens=(1000.0, 800.0, 900.0), phase_frac=0.5, box=(0.08, 0.08, 0.08))
    sc.params.mf_omega = 0.7
    sc.params.mf_visc_factor = 1.3
    out.append(("projectu_liquids", sc))
    return out


def main():
    O.build()
    if not O.ref_available():
        O.build_ref()
    for name, sc in fixtures():
        p = sc.params
        s = O.state_from_aos(sc.disp, sc.calc, p.gridtotal)
        s.bornid[:] = np.arange(s.n)  # the reference indexes MFidTable by bornid
        rec = {"params": np.frombuffer(bytes(p), np.uint8), "n": np.int64(s.n)}
        rec.update({"init_" + k: v for k, v in state_arrays(s).items()})
        for stage, fields in STAGES:
            if stage == "multiphase_inputs":
                prepare_multiphase(p, s, seed=zlib.crc32(name.encode()) % 1000)
            elif stage == "surface_tension" and not p.surface_tension:
                continue
            elif stage in SIDE_STAGES:
                t = s.copy()
                O.call_ref("ref_" + stage, p, t)
                for f in fields:
                    rec[f"{stage}__{f}"] = getattr(t, f).copy()
                continue
            else:
                O.call_ref("ref_" + stage, p, s)
            for f in fields:
                rec[f"{stage}__{f}"] = getattr(s, f).copy()
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **rec)
        print(f"{path}: n={s.n} ({os.path.getsize(path) // 1024} KiB)")
    with open(os.path.join(HERE, "README.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "source": "reference kernels compiled as host C++ (oracle/ref/build_ref.sh)",
                   "fixtures": [n for n, _ in fixtures()]}, f, indent=1)


if __name__ == "__main__":
    main()
