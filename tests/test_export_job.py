"""MeshExport's asynchronous job on the host (export.h:27-39, export.cpp:483-592): the
call returns at once, GetExportProgress reports the stage, one export runs at a time,
CancelExport(false) moves the stage word on as ExportState.fetch_add(1) does, and
CancelExport(true) halts the job -- here at its first stage, before it touches the GPU,
so no GPU is needed -- with no file written and the library ready for the next export."""

import pytest

from tangerine_gb300 import _lib, sdf

LO, HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


def test_export_job_pauses_reports_progress_and_halts(lib, tmp_path):
    t = sdf.sphere(0.5)
    path = tmp_path / "halted.ply"
    lib.tg_debug_export_pause(1)
    try:
        sdf.mesh_export(t, path, LO, HI, 0.1, 0, "ply", wait=False)
        assert lib.tg_debug_export_paused(10000) == 1
        stage, gen, ref, sec, wr = sdf.export_progress()
        assert (stage, gen, ref, sec, wr) == (1, 0.0, 0.0, 0.0, 0.0)
        # one export at a time: a second one is refused and the first keeps running
        with pytest.raises(_lib.TangerineError, match="already running"):
            sdf.mesh_export(t, tmp_path / "second.ply", LO, HI, 0.1, 0, "ply", wait=False)
        assert sdf.export_result(wait=False) == 8            # TG_ERR_BUSY
        sdf.cancel_export(False)                             # "good enough": ExportState += 1
        assert sdf.export_progress()[0] == 2
        sdf.cancel_export(True)                              # "halt"
        assert sdf.export_result(wait=True) == 7             # TG_ERR_CANCELLED
        assert b"halted" in lib.tg_last_error()
        assert sdf.export_progress()[0] == 0
        assert not path.exists() and not (tmp_path / "second.ply").exists()
    finally:
        lib.tg_debug_export_pause(0)
    assert sdf.export_result(wait=False) == 7                # the outcome stays readable


def test_export_arguments_are_checked_before_the_job_starts(lib, tmp_path):
    t = sdf.sphere(0.5)
    for kw, step in ((dict(fmt="vox"), 0.1), (dict(fmt="stl", point_cloud=True), 0.1), (dict(fmt="ply"), (0.1, 0.0, 0.1)),
                     (dict(fmt="ply"), -0.1)):
        with pytest.raises(_lib.TangerineError):
            sdf.mesh_export(t, tmp_path / "x", LO, HI, step, 0, wait=False, **kw)
        assert sdf.export_progress()[0] == 0                 # nothing started
    assert not (tmp_path / "x").exists()
