"""Disk I/O overlapped with GPU work for the file-driven drivers.

The reference drivers loop over the matching files of InputDir and, for each one,
read it, reconstruct (or project) it and write the result before touching the next
(run_mgfbp.py:52-85, run_mgfpj_v3.py:82-127).  run_over_files keeps that order and
those results but runs three stages concurrently: the read of file i+1 on a reader
thread and the write of file i-1 on a writer thread while the calling thread drives
the GPU for file i (numpy file reads and writes release the GIL).

The drivers' read and save methods keep the reference's signatures and set per-file
attributes on the driver (input/output paths, the loaded array; the save converts
the result in place, e.g. to HU).  So that the stages do not race on the driver, each
read and each save runs on a shallow copy of it; the attributes a read sets are moved
onto the driver when that file's turn comes, and after the last save its changes are
moved back, so the driver ends in the state the sequential loop leaves it in.
"""
import copy
from concurrent.futures import ThreadPoolExecutor


def _changes(before, obj):
    """Attributes of obj that are new or rebound since the snapshot `before`."""
    return {k: v for k, v in obj.__dict__.items() if k not in before or before[k] is not v}


def _read(c, before, method, file):
    ok = method(c, file)
    return ok, _changes(before, c)


def _submit_read(pool, driver, method, file):
    c = copy.copy(driver)  # taken on the calling thread, between its updates of the driver
    return pool.submit(_read, c, dict(c.__dict__), method, file)


def run_over_files(driver, files, read, compute, save):
    """For each file in order: `read(driver, file)` (returns False to skip the file),
    then `compute(driver)`, then `save(driver)`, with the read one file ahead and the
    save one file behind the compute.  An exception from any stage is raised here once
    the reads and saves already queued have finished; a failed save surfaces no later
    than the end of the next file's compute.  Returns the number of files computed."""
    files = list(files)
    done = 0
    with ThreadPoolExecutor(1, thread_name_prefix="mct-read") as rd, \
            ThreadPoolExecutor(1, thread_name_prefix="mct-write") as wr:
        nxt = _submit_read(rd, driver, read, files[0]) if files else None
        pending = None  # (future, copy, snapshot) of the last queued save
        for i in range(len(files)):
            ok, attrs = nxt.result()
            nxt = _submit_read(rd, driver, read, files[i + 1]) if i + 1 < len(files) else None
            if not ok:
                continue
            driver.__dict__.update(attrs)
            compute(driver)
            done += 1
            if pending is not None:
                pending[0].result()
            w = copy.copy(driver)
            snapshot = dict(w.__dict__)  # before the writer can touch w
            pending = (wr.submit(save, w), w, snapshot)
        if pending is not None:
            pending[0].result()
            driver.__dict__.update(_changes(pending[2], pending[1]))
    return done
