"""The autotuner's on-disk cache under concurrent writers (no GPU needed).

Several processes store tuning records at once through the cache's file
lock; the file must stay valid JSON holding every record (the read-modify-
write happens under an exclusive lock, the new file replaces the old
atomically)."""

import json
import multiprocessing as mp


def _writer(path, wid, n):
    import os

    os.environ["NLSE_AUTOTUNE_CACHE"] = path
    from nlse_gb300 import autotune

    for i in range(n):
        autotune._store(f"gpu|2d|{wid}x{i}", {"variant": [bool(i % 2), True],
                                              "ms_per_step": {"x": float(i)}})


def test_concurrent_writers_keep_every_record(tmp_path):
    path = str(tmp_path / "cache" / "autotune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(path, w, 15)) for w in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    with open(path) as f:
        data = json.load(f)
    assert set(data) == {f"gpu|2d|{w}x{i}" for w in range(4) for i in range(15)}
    assert data["gpu|2d|3x14"]["ms_per_step"]["x"] == 14.0


def test_unreadable_cache_reads_as_empty(tmp_path, monkeypatch):
    from nlse_gb300 import autotune

    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert autotune._read(str(p)) == {}
    monkeypatch.setenv("NLSE_AUTOTUNE_CACHE", str(p))
    autotune._store("k", {"variant": [True, True]})
    assert json.loads(p.read_text()) == {"k": {"variant": [True, True]}}
