"""Generates tests/golden/*.npz from the REFERENCE's own implementation.

The reference header src/pore_extraction.hpp is compiled unmodified against the project's Kokkos
shim (oracle/build_ref.sh -> oracle/_ref/libpnm_ref.so); this script runs it on seeded synthetic
inputs and stores the outputs (and, for inputs built from transcendental functions whose last
ulp may differ across platforms, the inputs themselves) as compressed fixtures. The fixtures pin
the project's C++ restatement (oracle/) on machines where the reference checkout is absent.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py NAME ...   # only these
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cases import random_volume  # noqa: E402
from oracle import Oracle, sorted_pores  # noqa: E402
from peclet_pnm_gb300 import synthetic as syn  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        if a is None:
            h.update(b"none")
        else:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


# name -> (builder, origin_zyx, spacing_zyx, store_input)
NETWORK_CASES = {
    "ci_lattice": (lambda: syn.ci_lattice(), [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], False),
    "sphere_lattice_36x30x24": (lambda: syn.sphere_lattice(36, 30, 24), [0.0, 0.0, 0.0],
                                [1.0, 1.0, 1.0], False),
    "trig_32_aniso": (lambda: syn.trig_field(32, 32, 32), [0.5, 2.0, -1.0], [2.0, 1.0, 0.5], True),
    "random_spheres_64": (lambda: syn.random_spheres(), [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], False),
    "chamber_tube": (lambda: syn.chamber_tube(), [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], False),
    "capsules": (lambda: syn.capsules(), [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], False),
    "packing_40x48x56": (lambda: syn.packing((40, 48, 56), 0.4, seed=7), [0.0, 0.0, 0.0],
                         [1.0, 1.0, 1.0], False),
}
# four of the seeded random volumes of tests/cases.py, one per value family (noise, quantised
# plateaus, noisy packing, marker-heavy), anisotropic spacing and offset origin; inputs stored
for _s in (20, 17, 31, 34):
    _sdf, _org, _spc = random_volume(_s)
    NETWORK_CASES[f"random_volume_{_s}"] = (lambda v=_sdf: v, _org, _spc, True)

# flow: (sdf builder, fields builder, origin_zyx, spacing_zyx, grad_p_zyx, with_openness)
FLOW_CASES = {
    "flow_lattice_open": (lambda: syn.sphere_lattice(36, 30, 24),
                          lambda s: syn.mac_fields(36, 30, 24), [2.0, -1.0, 0.5], [1.5, 1.0, 0.5],
                          [0.5e-3, -2e-3, 1e-3], True),
    "flow_lattice_fullyopen": (lambda: syn.sphere_lattice(36, 30, 24),
                               lambda s: syn.mac_fields(36, 30, 24), [2.0, -1.0, 0.5],
                               [1.5, 1.0, 0.5], [0.5e-3, -2e-3, 1e-3], False),
    "flow_capsules": (lambda: syn.capsules(), lambda s: syn.fourier_fields(s, seed=4),
                      [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.0, 0.0, -1e-3], True),
    "flow_packing_48": (lambda: syn.packing((48, 48, 48), 0.4, seed=3),
                        lambda s: syn.fourier_fields(s, seed=4), [0.0, 0.0, 0.0], [1.0, 1.0, 1.0],
                        [0.0, 0.0, -1e-4], True),
}


def main(names=None):
    ref = Oracle("reference")
    for name, (mk, org, spc, store) in NETWORK_CASES.items():
        if names and name not in names:
            continue
        sdf = np.ascontiguousarray(mk(), dtype=np.float32)
        pores, seg, pairs = ref.extract_pore_network(sdf, org, spc)
        staged = ref.extract_pores(sdf, org, spc)
        out = dict(origin=np.array(org), spacing=np.array(spc), shape=np.array(sdf.shape),
                   input_sha256=digest(sdf), pores=sorted_pores(pores), seg=seg, pairs=pairs,
                   staged_pores=sorted_pores(staged))
        if store:
            out["sdf"] = sdf
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: {len(pores)} pores, {len(pairs)} pairs")
    for name, (mk, mkf, org, spc, gp, opn) in FLOW_CASES.items():
        if names and name not in names:
            continue
        sdf = np.ascontiguousarray(mk(), dtype=np.float32)
        f = mkf(sdf)
        kw = dict(ox=f[4], oy=f[5], oz=f[6]) if opn else {}
        r = ref.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, **kw)
        out = dict(origin=np.array(org), spacing=np.array(spc), shape=np.array(sdf.shape),
                   grad_p=np.array(gp), with_openness=np.array(opn),
                   input_sha256=digest(sdf, *f[:4], *(f[4:] if opn else (None,))), **r)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: {len(r['pores'])} pores, {len(r['throats'])} throats")


if __name__ == "__main__":
    main(set(sys.argv[1:]) or None)
