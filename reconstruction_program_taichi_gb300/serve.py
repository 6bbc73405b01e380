"""Reconstruction serving loop on one GPU: continuous admission, same-geometry
batching, captured CUDA graphs, p50/p99 latency.

No counterpart in the reference (it reconstructs one config at a time).

Model
  * A request is an FBP/FDK reconstruction or an N-iteration CGLS solve of one
    sinogram for one geometry (a parsed config).
  * Requests of the same geometry and kind share a *slot class*.  A slot owns
    device buffers for up to `batch` requests, a CUDA stream, and a CUDA graph of
    the whole batch captured once (weight -> filter -> pack -> backproject for each
    sinogram, or the full CGLS loop), so a batch executes as one graph launch.
  * Admission is continuous: a scheduler thread takes pending requests in arrival
    order, groups those whose slot class matches (up to `batch`), and starts them on
    a free slot; new slots are created while the HBM budget allows, and a slot is
    reused as soon as its previous batch finishes.  Batches on different slots run
    concurrently on their own streams.
  * Slots are kept for reuse; when a request needs a new slot and the budget is
    spent, idle slots of other classes are evicted, least recently used first.
  * Inputs may be host arrays or CUDA tensors already resident on the device; the
    result comes back in the same form (a new device tensor for device inputs, so
    resident data never crosses the host link).  Inputs may also be file paths, read
    with the reference's conventions for the request's config on the server's I/O
    threads from the moment of submission; a request is admitted only once its
    inputs are in memory, so disk reads overlap the GPU work of other requests.  With
    `out_path` the result is also written there on an I/O thread after its slot has
    been released; the future resolves once the file is written.
  * Results do not depend on the mix: every kernel is deterministic and a slot's
    graph always runs the same kernels on the same buffer layout.
"""
import os
import queue
import threading
import time
from concurrent.futures import Future, ThreadPoolExecutor

import numpy as np
import torch

from . import ops
from .fbp import FdkPipeline
from .io import imwriteRaw, read_sinogram_file

_SENTINEL = object()


def _geom_key(obj, kind, extra=()):
    g = (obj.det_elem_count_horizontal, obj.det_elem_count_vertical_actual, obj.view_num, obj.img_dim,
         obj.img_dim_z, float(obj.det_elem_width), float(obj.det_elem_height), float(obj.img_pix_size),
         float(obj.img_voxel_height), float(obj.source_isocenter_dis), float(obj.source_det_dis),
         float(obj.total_scan_angle), float(obj.img_rot), bool(obj.cone_beam), bool(obj.curved_dect),
         str(obj.kernel_name), float(obj.kernel_param), float(obj.det_offset_horizontal),
         float(getattr(obj, "det_offset_vertical", 0.0)), float(obj.img_center_x), float(obj.img_center_y),
         float(obj.img_center_z), int(obj.recon_view_mode))
    return (kind,) + g + tuple(extra)


def _is_path(a):
    return isinstance(a, (str, os.PathLike))


def _input_error(r):
    """The exception of a failed input read of request r, else None."""
    for a in (r.sgm, r.x0):
        if isinstance(a, Future) and a.done() and a.exception() is not None:
            return a.exception()
    return None


def _inputs_ready(r):
    return all(not isinstance(a, Future) or a.done() for a in (r.sgm, r.x0))


def _resolve_inputs(r):
    if isinstance(r.sgm, Future):
        r.sgm = r.sgm.result()
    if isinstance(r.x0, Future):
        r.x0 = r.x0.result()


def _to_device(a, device):
    """A host array or a tensor as a float32 tensor on device (no copy when it already is)."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float32)
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(device)


class _Request:
    __slots__ = ("kind", "obj", "sgm", "x0", "n_iter", "storage", "key", "future", "t_arrive", "t_start",
                 "t_done", "units", "on_device", "out_path")

    def __init__(self, kind, obj, sgm, x0=None, n_iter=0, storage="f32", out_path=None):
        self.kind, self.obj, self.sgm, self.x0, self.n_iter, self.storage = kind, obj, sgm, x0, n_iter, storage
        self.out_path = out_path
        extra = (storage, n_iter) if kind == "cgls" else (storage,)
        self.key = _geom_key(obj, kind, extra)
        self.future = Future()
        self.t_arrive = time.perf_counter()
        self.t_start = self.t_done = None
        nvox = obj.img_dim * obj.img_dim * obj.img_dim_z
        self.units = nvox * obj.view_num * (1 if kind == "fbp" else 2 * (n_iter + 1))
        self.on_device = isinstance(sgm, torch.Tensor) and sgm.is_cuda


class _FbpSlot:
    """Static buffers and one captured graph for `batch` FBP reconstructions."""

    def __init__(self, obj, batch, storage, device, use_graph):
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.batch = batch
        with torch.cuda.stream(self.stream):
            self.pipes = [FdkPipeline(obj, device=device, storage=storage) for _ in range(batch)]
            shape = self.pipes[0].dg.sgm_shape
            self.inp = [torch.zeros(shape, dtype=torch.float32, device=device) for _ in range(batch)]
            self.out = [torch.zeros(self.pipes[0].dg.vol_shape, dtype=torch.float32, device=device)
                        for _ in range(batch)]
        self.host_out = [torch.empty(self.pipes[0].dg.vol_shape, dtype=torch.float32, pin_memory=True)
                         for _ in range(batch)]
        self.graph = None
        self.last_used = time.perf_counter()
        self.nbytes = sum(p.weighted.numel() * 4 + p.filtered.numel() * 4 + p.packed.numel() + p.vol.numel() * 4
                          + (p.tc._buf.numel() if p.tc is not None else 0)
                          for p in self.pipes) + sum(t.numel() * 4 for t in self.inp + self.out)
        if use_graph:
            self._capture()

    def _body(self):
        for p, i, o in zip(self.pipes, self.inp, self.out):
            p.run(i, out=o)

    def _capture(self):
        with torch.cuda.stream(self.stream):
            self._body()  # warm (first-call set-up outside the capture)
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        # thread-local capture: other slots keep running on their own threads/streams
        with torch.cuda.graph(g, stream=self.stream, capture_error_mode="thread_local"):
            self._body()
        self.graph = g

    def run(self, reqs):
        dev_out = []
        with torch.cuda.stream(self.stream):
            for i, r in enumerate(reqs):
                if r.on_device:
                    self.inp[i].copy_(r.sgm)
                else:
                    self.inp[i].copy_(torch.from_numpy(np.ascontiguousarray(r.sgm, dtype=np.float32)))
            if self.graph is not None:
                self.graph.replay()
            else:
                self._body()
            for i, r in enumerate(reqs):
                if r.on_device:
                    dev_out.append(self.out[i].clone())
                else:
                    dev_out.append(None)
                    self.host_out[i].copy_(self.out[i], non_blocking=True)
        self.stream.synchronize()
        self.last_used = time.perf_counter()
        return [d if d is not None else self.host_out[i].numpy().copy() for i, d in enumerate(dev_out)]


def _fp_workspace_bytes(dg):
    from . import _lib
    return int(_lib.load().mct_fp_storage_workspace_size(dg.g(), _lib.MCT_F32))


class _CglsSlot:
    """CGLS (reference operator pair, lambda*D^T D with unit weights) for one request."""

    def __init__(self, obj, n_iter, device):
        from .ir import IrSystem
        self.stream = torch.cuda.Stream(device=device)
        self.batch = 1
        with torch.cuda.stream(self.stream):
            self.sys = IrSystem(obj, device)
        self.obj = obj
        self.n_iter = n_iter
        self.last_used = time.perf_counter()
        nvol = obj.img_dim * obj.img_dim * obj.img_dim_z
        # iterates and operator buffers, the projector's gather copies, sinogram buffers
        self.nbytes = 4 * nvol * 4 + _fp_workspace_bytes(self.sys.dg) + 3 * self.sys.fp_buf.numel() * 4

    def run(self, reqs):
        r = reqs[0]
        obj = self.obj
        with torch.cuda.stream(self.stream):
            sgm = _to_device(r.sgm, self.sys.device)
            x0 = _to_device(r.x0, self.sys.device)
            self.sys.bpb = self.sys.bp_b(sgm)
            wr = torch.ones_like(x0)
            lr = obj.coef_lambda * obj.pixel_count_ratio
            x = self.sys.cgls(x0, [], [(lr, wr)], self.n_iter)
            out = x if r.on_device else x.cpu().numpy()
        self.stream.synchronize()
        self.last_used = time.perf_counter()
        return [out]


class ReconServer:
    """Continuous-batching reconstruction server on one GPU (see module docstring)."""

    def __init__(self, device=None, hbm_budget_gb=150.0, batch=4, max_slots_per_class=4, use_graphs=True):
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required")
        self.device = torch.device(device or "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.budget = int(hbm_budget_gb * 1e9)
        self.used = 0
        self.batch = batch
        self.max_slots = max_slots_per_class
        self.use_graphs = use_graphs
        self.pending = []
        self.cv = threading.Condition()
        self.free_slots = {}    # key -> [slot]
        self.all_slots = {}     # key -> count
        self.evictions = 0
        self.busy = 0
        self.done = []
        self.closed = False
        self.errors = []
        self._workers = []
        self._io = ThreadPoolExecutor(2, thread_name_prefix="mct-serve-io")
        self._thread = threading.Thread(target=self._schedule, daemon=True)
        self._thread.start()

    # ------------------------------------------------------------ API
    def submit_fbp(self, obj, sgm, storage="f32", out_path=None):
        """FBP/FDK of a sinogram [rows, views, cols] (host array, CUDA tensor, or the path
        of an input file in the config's InputFileForm and detector row range) for the
        parsed config obj; the future's result is a host array or a new CUDA tensor.
        out_path: also write the result there (raw float32)."""
        sgm = self._load(sgm, lambda p: read_sinogram_file(obj, p))
        return self._submit(_Request("fbp", obj, sgm, storage=storage, out_path=out_path))

    def submit_cgls(self, obj, sgm, x0, n_iter, out_path=None):
        """n_iter CGLS iterations (Tikhonov-TV with unit weights) from x0 (host arrays,
        CUDA tensors or file paths as for submit_fbp; a volume file is raw float32
        [z, y, x])."""
        sgm = self._load(sgm, lambda p: read_sinogram_file(obj, p))
        x0 = self._load(x0, lambda p: np.fromfile(p, dtype=np.float32).reshape(obj.img_dim_z, obj.img_dim,
                                                                             obj.img_dim))
        return self._submit(_Request("cgls", obj, sgm, x0=x0, n_iter=n_iter, out_path=out_path))

    def close(self, wait=True):
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        if wait:
            self._thread.join()
            for t in self._workers:
                t.join()
        self._io.shutdown(wait=wait)  # pending result writes finish first when waiting

    def stats(self):
        """Latency (arrival to result), its queueing and service parts, throughput."""
        done = list(self.done)
        lat = np.array([(r.t_done - r.t_arrive) * 1e3 for r in done]) if done else np.zeros(1)
        wait = np.array([(r.t_start - r.t_arrive) * 1e3 for r in done]) if done else np.zeros(1)
        serv = np.array([(r.t_done - r.t_start) * 1e3 for r in done]) if done else np.zeros(1)
        t0 = min(r.t_arrive for r in done) if done else 0.0
        t1 = max(r.t_done for r in done) if done else 1.0
        units = sum(r.units for r in done)
        slots = {}
        for k, v in self.all_slots.items():
            slots[k[0]] = slots.get(k[0], 0) + v
        return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "queue_p50_ms": float(np.percentile(wait, 50)), "service_p50_ms": float(np.percentile(serv, 50)),
                "service_p99_ms": float(np.percentile(serv, 99)),
                "gups": units / max(t1 - t0, 1e-9) / 1e9, "slots": slots, "classes": len(self.all_slots),
                "evictions": self.evictions, "hbm_used_gb": self.used / 1e9}

    # ------------------------------------------------------------ internals
    def _load(self, a, reader):
        """A path becomes a future of its contents, read on an I/O thread; the scheduler
        is woken when the read ends."""
        if not _is_path(a):
            return a
        fut = self._io.submit(reader, os.fspath(a))
        fut.add_done_callback(self._wake)
        return fut

    def _wake(self, _fut=None):
        with self.cv:
            self.cv.notify_all()

    def _write_result(self, r, out):
        try:
            imwriteRaw(out.cpu().numpy() if isinstance(out, torch.Tensor) else out, os.fspath(r.out_path),
                       dtype=np.float32)
            r.future.set_result(out)
        except Exception as e:  # noqa: BLE001 - handed to the caller through the future
            r.future.set_exception(e)

    def _submit(self, req):
        with self.cv:
            if self.closed:
                raise RuntimeError("server is closed")
            self.pending.append(req)
            self.cv.notify_all()
        return req.future

    def _make_slot(self, req):
        torch.cuda.set_device(self.device)
        if req.kind == "fbp":
            return _FbpSlot(req.obj, self._batch_for(req), req.storage, self.device, self.use_graphs)
        return _CglsSlot(req.obj, req.n_iter, self.device)

    @staticmethod
    def _per_request_bytes(req):
        o = req.obj
        nvol = o.img_dim * o.img_dim * o.img_dim_z * 4
        nsgm = o.det_elem_count_horizontal * o.det_elem_count_vertical_actual * o.view_num * 4
        if req.kind == "fbp":  # input, weighted, filtered, packed (4x), tensor-core operand tiles
            return nsgm * 8 + 2 * nvol
        # CGLS: four iterates, the projector's gather copies (cone beam: two 32-byte cells
        # per voxel), three sinogram buffers
        return 4 * nvol + (16 if o.cone_beam else 1) * nvol + 3 * nsgm

    def _batch_for(self, req):
        """Requests per FBP slot: `batch`, reduced so that one slot takes at most an
        eighth of the budget (large geometries get small slots, so that several classes
        stay resident)."""
        if req.kind != "fbp":
            return 1
        return max(1, min(self.batch, int(self.budget / 8 // max(self._per_request_bytes(req), 1))))

    def _estimate(self, req):
        return self._batch_for(req) * self._per_request_bytes(req)

    def _schedule(self):
        while True:
            with self.cv:
                while not self.closed and not self.pending:
                    self.cv.wait()
                if self.closed and not self.pending:
                    break
                started = self._try_start()
                if not started:
                    self.cv.wait(timeout=0.05)

    def _try_start(self):
        """Start the oldest pending request's class if a slot is free or can be
        created within the budget; returns True if something started."""
        for i, head in enumerate(self.pending):
            err = _input_error(head)
            if err is not None:  # its input file could not be read: fail this request only
                head.future.set_exception(err)
                self.pending.pop(i)
                return True
            if not _inputs_ready(head):
                continue
            key = head.key
            free = self.free_slots.setdefault(key, [])
            slot = free.pop() if free else None
            if slot is None:
                if self.all_slots.get(key, 0) >= self.max_slots:
                    continue
                need = self._estimate(head)
                if self.used + need > self.budget:
                    self._evict_idle(need, keep=key)
                if self.used + need > self.budget:
                    if self.busy == 0 and not any(self.free_slots.values()):
                        head.future.set_exception(MemoryError("request exceeds the HBM budget"))
                        self.pending.pop(i)
                        return True
                    continue
                try:
                    slot = self._make_slot(head)
                except Exception as e:  # allocation or build failure: fail this request only
                    head.future.set_exception(e)
                    self.pending.pop(i)
                    return True
                self.used += slot.nbytes
                self.all_slots[key] = self.all_slots.get(key, 0) + 1
            group = [r for r in self.pending if r.key == key and _inputs_ready(r) and _input_error(r) is None]
            group = group[:slot.batch]
            for r in group:
                self.pending.remove(r)
                r.t_start = time.perf_counter()
            self.busy += 1
            t = threading.Thread(target=self._run, args=(slot, key, group), daemon=True)
            self._workers.append(t)
            t.start()
            return True
        return False

    def _evict_idle(self, need, keep):
        """Release idle slots of other classes, least recently used first, until `need`
        bytes fit in the budget (called with the lock held)."""
        idle = [(s.last_used, k, s) for k, lst in self.free_slots.items() if k != keep for s in lst]
        for _, k, s in sorted(idle, key=lambda t: t[0]):
            if self.used + need <= self.budget:
                break
            self.free_slots[k].remove(s)
            self.all_slots[k] -= 1
            if self.all_slots[k] == 0:
                del self.all_slots[k]
            self.used -= s.nbytes
            self.evictions += 1
            del s

    def _run(self, slot, key, group):
        outs, err = None, None
        try:
            torch.cuda.set_device(self.device)
            for r in group:
                _resolve_inputs(r)
            outs = slot.run(group)
            now = time.perf_counter()
            for r in group:
                r.t_done = now
        except Exception as e:  # a failed batch fails its own requests only
            err = e
            self.errors.append(e)
        # record completion and free the slot before any caller can observe the result
        with self.cv:
            if outs is not None:
                self.done.extend(group)
            self.busy -= 1
            self.free_slots.setdefault(key, []).append(slot)
            self.cv.notify_all()
        for i, r in enumerate(group):
            if outs is not None:
                if r.out_path is not None:
                    try:
                        self._io.submit(self._write_result, r, outs[i])
                    except RuntimeError:  # I/O threads already shut down (close without waiting)
                        self._write_result(r, outs[i])
                else:
                    r.future.set_result(outs[i])
            elif not r.future.done():
                r.future.set_exception(err)
