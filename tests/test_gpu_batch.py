"""Many trees in one persistent launch: every model's mesh must equal the single-model
export of its program and lattice, bit for bit, whatever the per-model tuning."""

import numpy as np
import pytest

from tangerine_gb300 import sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MODELS = [(11, 4, 24), (12, 16, 40), (17, 64, 32), (14, 256, 48), (15, 8, 16), (16, 128, 36)]


@pytest.fixture(scope="module")
def programs(lib):
    progs, grids = [], []
    for seed, prims, res in MODELS:
        ops = W.OPS_UNIFORM4 if prims <= 16 else W.OPS_60_20_10_10
        progs.append(sdf.compile(sdf.from_spec(W.random_tree(seed, prims, ops=ops))))
        grids.append(W.export_grid(resolution=res))
    # An unpainted tree too: the batch must leave its colours out as the export does.
    progs.append(sdf.compile(sdf.union(sdf.sphere(0.5), sdf.box(0.3, 0.4, 0.2).move(0.4, 0.0, 0.0))))
    grids.append(W.export_grid(resolution=20))
    yield progs, grids
    for p in progs:
        p.close()


def _same(a, b):
    np.testing.assert_array_equal(a.vertices, b.vertices)
    np.testing.assert_array_equal(a.faces, b.faces)
    np.testing.assert_array_equal(a.normals, b.normals)
    np.testing.assert_array_equal(a.cubes, b.cubes)
    assert (a.colors is None) == (b.colors is None)
    if a.colors is not None:
        np.testing.assert_array_equal(a.colors, b.colors)


def test_batch_meshes_equal_single_exports(programs):
    progs, grids = programs
    singles = [p.export_mesh(g) for p, g in zip(progs, grids)]
    with sdf.Batch(progs, grids) as b:
        b.run()
        info = b.info()
        assert info.models == len(progs) and info.reruns == 0
        for m, ref in enumerate(singles):
            _same(b.mesh(m), ref)
        assert info.vertices == sum(len(r.vertices) for r in singles)
        assert info.faces == sum(len(r.faces) for r in singles)
        # Replay (from the CUDA graph when capture was accepted) gives the same again.
        b.run()
        assert b.info().graph in (1, -1)
        for m, ref in enumerate(singles):
            _same(b.mesh(m), ref)


def test_batch_mixed_tuning_and_growth(programs):
    progs, grids = programs
    singles = [p.export_mesh(g) for p, g in zip(progs, grids)]
    rng = np.random.default_rng(5)
    with sdf.Batch(progs, grids) as b:
        b.set_tuning(rng.choice([1, 3, 4, 7, 11, 15], len(progs)), rng.choice([1, 2, 4], len(progs)))
        b.reserve(64, 64)                 # far too small: the run grows the outputs and repeats
        b.run()
        assert b.info().reruns >= 1
        for m, ref in enumerate(singles):
            _same(b.mesh(m), ref)


def test_batch_autotune(programs):
    progs, grids = programs
    with sdf.Batch(progs[:3], grids[:3]) as b:
        b.autotune()
        bricks, lanes = b.tuning()
        assert set(bricks) <= {4, 7, 11, 15} and set(lanes) <= {1, 2, 4}
        b.run()
        for m in range(3):
            _same(b.mesh(m), progs[m].export_mesh(grids[m]))


def test_batch_surrogate_form_same_meshes(programs):
    """Learned bounds culling some models' bricks inside the batch (with and without the exact
    test of the kept bricks, a model without a network in between): every mesh is still the
    exact export's."""
    progs, grids = programs
    singles = [p.export_mesh(g) for p, g in zip(progs, grids)]
    nets = []
    for m, p in enumerate(progs):
        if m in (1, 3, 5):
            s = sdf.Surrogate(samples=1 << 20, steps=400, batch=1 << 16, validation=1 << 18)
            s.fit(p)
            nets.append(s)
        else:
            nets.append(None)
    try:
        with sdf.Batch(progs, grids) as b:
            b.set_tuning(bricks=[7, 4, 7, 5, 3, 7, 2])
            refined_bricks = None
            for only in (False, True):
                b.set_surrogates(nets, only=only)
                b.run()
                info = b.info()
                for m, ref in enumerate(singles):
                    _same(b.mesh(m), ref)
                if not only:
                    refined_bricks = info.bricks_evaluated
            b.set_surrogates([None] * len(progs))
            b.run()
            # The exact test alone keeps at least what the network and the exact test keep.
            assert b.info().bricks_evaluated >= refined_bricks
            for m, ref in enumerate(singles):
                _same(b.mesh(m), ref)
    finally:
        for s in nets:
            if s is not None:
                s.close()


def test_batch_cancel_and_barrier_time_limit(lib, programs):
    """Failure paths of the persistent kernel, made on purpose with no GPU fault: a cancel
    flag set on the host ends the run at its first grid barrier (TG_ERR_CANCELLED, every
    block gone); a block started 300 ms late makes the other blocks' 20 ms barrier wait run
    out (TG_ERR_CUDA, "timed out", every block gone).  After each, the context is usable
    and the next run gives the same meshes as before."""
    progs, grids = programs
    singles = [p.export_mesh(g) for p, g in zip(progs, grids)]
    with sdf.Batch(progs, grids) as b:
        b.run()
        assert lib.tg_batch_cancel(b.ptr, 1) == 0
        assert lib.tg_batch_run(b.ptr, None) == 7
        assert b"cancelled" in lib.tg_last_error()
        b.run()                                    # the flag was cleared by the cancelled run
        for m, ref in enumerate(singles):
            _same(b.mesh(m), ref)
        assert lib.tg_batch_cancel(b.ptr, 1) == 0
        assert lib.tg_batch_cancel(b.ptr, 0) == 0  # withdrawn before the run
        b.run()
        assert lib.tg_batch_debug_barrier(b.ptr, 20_000_000, 0, 300_000_000) == 0
        assert lib.tg_batch_run(b.ptr, None) == 3
        assert b"timed out" in lib.tg_last_error()
        assert lib.tg_batch_debug_barrier(b.ptr, 0, -1, 0) == 0
        b.run()
        for m, ref in enumerate(singles):
            _same(b.mesh(m), ref)
        assert lib.tg_batch_debug_barrier(b.ptr, 0, 0, 3_000_000_000) != 0     # late start above 2 s refused
