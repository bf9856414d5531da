"""Output: snapshots of a problem's fields, its set-up and diagnostics (src/output.jl).

The reference writes JLD2 (a Julia HDF5 dialect).  This host writes the same keys —
``snapshots/t/<step>``, ``snapshots/<field>/<step>``, ``grid/...``, ``params/...``,
``clock/dt``, ``eqn/L``, ``eqn/dims``, ``eqn/T``, ``diagnostics/<name>/{steps,t,data}`` —
into a zip of ``.npy`` members (numpy's ``.npz`` container, appended to in place), and
``openoutput(path)`` reads it back as nested dictionaries, as ``jldopen`` would.

``saveoutput`` does not stall the time stepping: each device field is snapshotted by a
device-to-device copy on the current stream, the snapshot is copied into pinned host
memory on a side stream, and a writer thread appends it to the file once that copy's
event has completed.  ``flush(out)`` (or ``out.flush()``) waits for every pending write.
"""
from __future__ import annotations

import io
import os
import queue
import threading
import zipfile

import numpy as np

from .devices import on_device

EXT = ".npz"


def withoutjld2(path):
    """src/output.jl:32: `path` without a trailing ".jld2"."""
    return path[:-5] if len(path) > 4 and path[-5:] == ".jld2" else path


def _without_ext(path, ext):
    return path[:-len(ext)] if len(path) > len(ext) and path.endswith(ext) else path


def uniquepath(path):
    """src/output.jl:39-52: `path` with _1, _2, ... inserted before its extension until
    no such file exists (the extension is the path's own: ".jld2" in the reference)."""
    ext = os.path.splitext(path)[1] or ".jld2"
    n = 1
    if os.path.isfile(path):
        path = _without_ext(path, ext) + f"_{n}{ext}"
    while os.path.isfile(path):
        n += 1
        path = _without_ext(path, ext)[:-len(f"_{n - 1}")] + f"_{n}{ext}"
    return path


# ----------------------------------------------------------------------------------------
# the container and its writer
# ----------------------------------------------------------------------------------------
def _npy_bytes(a):
    buf = io.BytesIO()
    np.save(buf, np.asarray(a), allow_pickle=False)
    return buf.getvalue()


class _Writer:
    """One thread per file: appends (key, array) members in submission order."""

    def __init__(self, path):
        self.path = path
        self.q = queue.Queue()
        self.err = None
        self.t = threading.Thread(target=self._run, name=f"output:{os.path.basename(path)}", daemon=True)
        self.t.start()

    def _run(self):
        while True:
            item = self.q.get()
            try:
                if item is None:
                    return
                event, entries = item
                if event is not None:
                    event.synchronize()
                with zipfile.ZipFile(self.path, "a", compression=zipfile.ZIP_STORED) as z:
                    for key, arr in entries:
                        z.writestr(key + ".npy", _npy_bytes(arr.get() if isinstance(arr, _LazyHost) else arr))
            except Exception as e:  # reported by flush()
                self.err = e
            finally:
                self.q.task_done()

    def submit(self, event, entries):
        self.q.put((event, entries))

    def flush(self):
        self.q.join()
        if self.err is not None:
            e, self.err = self.err, None
            raise RuntimeError(f"writing {self.path} failed: {e}") from e


_writers = {}
_writers_lock = threading.Lock()


def _writer(path):
    path = os.path.abspath(path)
    with _writers_lock:
        w = _writers.get(path)
        if w is None:
            w = _writers[path] = _Writer(path)
        return w


def flush(target=None):
    """Wait for the pending writes of one Output (or path), or of all files."""
    if target is None:
        with _writers_lock:
            ws = list(_writers.values())
    else:
        path = target.path if isinstance(target, Output) else target
        ws = [_writer(path)]
    for w in ws:
        w.flush()


def _host_now(x):
    """A host copy of x (a device tensor, host tensor, numpy array or scalar)."""
    if on_device(x):
        from .devices import to_numpy
        return to_numpy(x)
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _write_now(path, entries):
    w = _writer(path)
    w.submit(None, [(k, _host_now(v)) for k, v in entries])
    w.flush()


# ----------------------------------------------------------------------------------------
# Output
# ----------------------------------------------------------------------------------------
class Output:
    """Output(prob, path, (name, func), ...) or Output(prob, path, {name: func})
    (src/output.jl:8-29).  The file is ``uniquepath`` of `path` with the ".npz"
    container suffix in place of ".jld2"."""

    def __init__(self, prob, path, *fields):
        if len(fields) == 1 and isinstance(fields[0], dict):
            fd = dict(fields[0])
        else:
            fd = {}
            for f in fields:
                name, func = f
                fd[name] = func
        self.prob = prob
        self.path = uniquepath(_without_ext(withoutjld2(path), EXT) + EXT)
        self.fields = {str(k).lstrip(":"): v for k, v in fd.items()}

    def __getitem__(self, key):
        """src/output.jl:54: the field computed now."""
        return self.fields[str(key).lstrip(":")](self.prob)

    def flush(self):
        flush(self)

    def __repr__(self):
        return ("Output\n"
                f"  ├──── prob: {type(self.prob).__name__}\n"
                f"  ├──── path: {self.path}\n"
                f"  └── fields: {{{', '.join(self.fields)}}}")


def saveoutput(out, stream=None):
    """src/output.jl:61-71: snapshots/t/<step> and snapshots/<field>/<step>.  A device
    field is first copied on the current stream into a private device buffer (a few
    microseconds at HBM speed, so later steps may overwrite the field at once), then
    copied to pinned host memory on a side stream; the file is written by the writer
    thread when that copy completes.  Returns without waiting."""
    step = int(out.prob.clock.step)
    entries = [(f"snapshots/t/{step}", np.asarray(float(out.prob.clock.t)))]
    event = None
    pending = []
    for name in out.fields:
        val = out[name]
        key = f"snapshots/{name}/{step}"
        if on_device(val):
            pending.append((key, val))
        else:
            entries.append((key, _host_now(val)))
    if pending:
        import torch
        cur = torch.cuda.current_stream() if stream is None else stream
        side = _side_stream()
        snaps = []
        with torch.cuda.stream(cur):
            for key, val in pending:
                snap = torch.empty_strided(val.shape, val.stride(), dtype=val.dtype, device=val.device)
                snap.copy_(val)
                snaps.append((key, snap))
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            for key, snap in snaps:
                host = torch.empty_strided(snap.shape, snap.stride(), dtype=snap.dtype, pin_memory=True)
                host.copy_(snap, non_blocking=True)
                snap.record_stream(side)
                entries.append((key, _LazyHost(host)))
            event = torch.cuda.Event()
            event.record(side)
    _writer(out.path).submit(event, entries)
    return None


class _LazyHost:
    """A pinned host tensor whose copy completes at its item's event."""

    def __init__(self, t):
        self.t = t

    def get(self):
        return self.t.numpy()


_side = None


def _side_stream():
    global _side
    if _side is None:
        import torch
        _side = torch.cuda.Stream()
    return _side


# ----------------------------------------------------------------------------------------
# saveproblem / savediagnostic (src/output.jl:80-161)
# ----------------------------------------------------------------------------------------
def _grid_entries(grid):
    from .domains import OneDGrid, ThreeDGrid, TwoDGrid
    if isinstance(grid, TwoDGrid):
        names = ["nx", "ny", "Lx", "Ly", "x", "y"]
    elif isinstance(grid, OneDGrid):
        names = ["nx", "Lx", "x"]
    elif isinstance(grid, ThreeDGrid):
        names = ["nx", "ny", "nz", "Lx", "Ly", "Lz", "x", "y", "z"]
    else:
        return []
    return [(f"grid/{n}", getattr(grid, n)) for n in names]


def _params_entries(params):
    out = []
    for name, field in vars(params).items():
        if callable(field) or type(field).__name__ in ("RFFTPlan", "FFTPlan"):
            continue  # forbidden_output_types (src/output.jl:104)
        try:
            arr = _host_now(field)
        except Exception:
            continue
        if arr.dtype == object:
            continue
        out.append((f"params/{name}", arr))
    return out


def saveproblem(prob, filename=None):
    """saveproblem(prob, filename) / saveproblem(out): eqn, clock, grid and params
    (src/output.jl:134-145); written before it returns."""
    if isinstance(prob, Output):
        prob, filename = prob.prob, prob.path
    entries = [("eqn/L", prob.eqn.L), ("eqn/dims", np.asarray(prob.eqn.dims, dtype=np.int64)),
               ("eqn/T", np.asarray(np.dtype(prob.eqn.T).name)), ("clock/dt", np.asarray(float(prob.clock.dt)))]
    entries += _grid_entries(prob.grid) + _params_entries(prob.params)
    _write_now(filename, entries)


def savediagnostic(diagnostic, diagname, filename):
    """src/output.jl:153-161: the computed part (through diagnostic.i) of steps, t, data."""
    i = diagnostic.i
    data = [_host_now(d) for d in diagnostic.data[:i]]
    try:
        data_arr = np.stack(data)
    except ValueError:
        data_arr = np.asarray(data, dtype=object)
    entries = [(f"diagnostics/{diagname}/steps", np.asarray(diagnostic.steps[:i], dtype=np.int64)),
               (f"diagnostics/{diagname}/t", np.asarray(diagnostic.t[:i], dtype=np.float64)),
               (f"diagnostics/{diagname}/data", data_arr)]
    _write_now(filename, entries)


def openoutput(path):
    """The file as nested dictionaries of numpy arrays (jldopen's group view):
    f["snapshots"]["c"]["0"]."""
    flush(path)
    root = {}
    with zipfile.ZipFile(path) as z:
        for name in z.namelist():
            key = name[:-4] if name.endswith(".npy") else name
            parts = key.split("/")
            d = root
            for p in parts[:-1]:
                d = d.setdefault(p, {})
            d[parts[-1]] = np.load(io.BytesIO(z.read(name)), allow_pickle=False)
    return root
