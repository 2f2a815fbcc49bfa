"""Batched box reconstructions in one CUDA graph: every mock's shifted
positions equal those of the same mock reconstructed alone through the
per-mock API (mixed meshes, boxes, CIC/TSC and smoothing radii), and a
replay reproduces them.  One CIC and one TSC mock are also checked against
the oracle pipeline (src/recon.jl:134-153 with src/iterative.jl,
src/mas.jl:218-269, src/recon.jl:264-388), so an error shared by the batch
and the per-mock path cannot hide."""
import numpy as np
import pytest

import baorec_oracle as O

pytestmark = pytest.mark.gpu

SPECS = [  # mesh, box, mas, R, particles, seed
    (32, 500.0, "cic", 12.0, 20000, 1),
    (64, 1000.0, "tsc", 15.0, 50000, 2),
    (32, 500.0, "tsc", 10.0, 15000, 3),
    (64, 1000.0, "cic", 13.0, 40000, 4),
]


def test_batch_matches_single_mock_reconstructions():
    import torch
    import baorec
    from baorec import mocks
    cat = [mocks.box_mock(n_part=np_, L=L, n_grid=n, seed=s) for n, L, _, _, np_, s in SPECS]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    items, outs = [], []
    for (n, L, mas, R, np_, _), m in zip(SPECS, cat):
        o = tuple(torch.empty(np_, device="cuda") for _ in range(3))
        outs.append(o)
        items.append(dict(x=dev(m.x), y=dev(m.y), z=dev(m.z), w=dev(m.w), mesh=n, box_size=L, mas=mas,
                          smoothing_radius=R, field="sum", out=o))
    base = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, los=[0.0, 0.0, 1.0], n_iter=3)
    b = baorec.Batch(base, items)
    b.launch()
    b.sync()
    first = [tuple(t.cpu().numpy().copy() for t in o) for o in outs]
    for t3 in outs:
        for t in t3:
            t.zero_()
    b.launch()
    b.sync()
    assert b.kernel_launches() > 0
    for (n, L, mas, R, np_, _), m, o, f0 in zip(SPECS, cat, outs, first):
        rec = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=R, box_size=[L] * 3, box_min=[0.0] * 3,
                                    los=[0.0, 0.0, 1.0], n_iter=3, mas=mas)
        delta = baorec.zeros_mesh((n, n, n), device=False)
        x, y, z = m.x.copy(), m.y.copy(), m.z.copy()
        baorec.reconstructed_overdensity_(delta, rec, x, y, z, m.w)
        ref = baorec.reconstructed_positions(rec, x, y, z, delta, field="sum")
        for a in range(3):
            got = o[a].cpu().numpy()
            # float atomics in the paint may add in another order: Mpc/h-level agreement far below 1e-3
            assert np.max(np.abs(got - np.asarray(ref[a]))) < 1e-3
            assert np.max(np.abs(got - f0[a])) < 1e-3
    # the oracle pipeline for the first CIC and the first TSC mock
    for i in (0, 1):
        n, L, mas, R, np_, _ = SPECS[i]
        m = cat[i]
        d, _, _, pos = O.run_iterative((n,) * 3, 2.0, 0.8, R, m.x, m.y, m.z, m.w, box_size=[L] * 3,
                                       box_min=[0.0] * 3, los=[0.0, 0.0, 1.0], n_iter=3, mas=mas)
        disp = O.compute_displacements_iterative(d, *pos, [L] * 3, [0.0] * 3)
        ref = O.reconstructed_positions(O.read_shifts(disp, *pos, 0.8, los=[0.0, 0.0, 1.0], field="sum"), *pos)
        for a in range(3):
            assert np.max(np.abs(outs[i][a].cpu().numpy() - ref[a])) < 1e-3, (i, a)
    b.close()
