"""Step checkpoints of a ``PIC_loop``: save the whole state of a run, restore
it later, and recompute from it.

The reference has no restart facility (its HDF5 records are write-only,
chimeraCL/diagnostics.py:57-78).  A checkpoint here holds everything the
following steps read:

* every ``DataDev`` tensor of the loop's solvers and species (cloned on the
  device; working buffers and caches whose names start with ``_`` and the
  transforms' scratch buffers are left out -- they are rewritten before
  they are read);
* the host ``Args`` of each solver and species (numpy arrays copied, the
  lazily read device scalars -- in-window count, injector right limit --
  resolved; links to other objects, such as the ions' ``InjectorSource``,
  marked and left to the run), and each species' ``flag_sorted``;
* each species' injector random-number generator state (the draws of the
  next window shifts);
* the loop's step count.

``restore_checkpoint`` puts that state back: into each ``DataDev`` tensor in
place where the run's tensor has the saved shape and type (the loop's CUDA
graphs, whose launches name those buffers, then stay valid: a restored step
between the same window shifts replays instead of capturing again), else by
rebinding the entry to a fresh copy; the checkpoint itself is never handed
out, so it can be restored again.  A run
restored to step n and stepped to step m reproduces, bit for bit, the run
that went from n to m before (the kernels are deterministic), which is
what a recompute-from-checkpoint scheme needs.

``state_dict`` / ``load_state_dict`` move a checkpoint to host memory and
back, so that ``torch.save`` can write it (``torch.load`` it with
``weights_only=False``: it holds numpy arrays and generator states)."""
import copy

import numpy as np
import torch

from .methods.generic_methods_cu import LazyScalar

SCRATCH_PREFIXES = ("_", "buff_fb", "fld_buff")
# entries that only name another entry's buffer (the solver's current phase
# factors): not saved, and set again by the code that uses them
ALIASES = ("phs_shft",)
# host values a checkpoint stores; anything else in Args (an object such as
# the ions' InjectorSource species) is a link the run keeps: marked, not
# copied, and left as it is on restore
_PLAIN = (bool, int, float, complex, str, bytes, type(None), np.ndarray, np.generic, list,
          dict, tuple)


class _Live:
    """Marks an Args entry that a restore leaves as it is."""

    def __repr__(self):
        return "<kept by the run>"


LIVE = _Live()


def _is_scratch(key):
    return key.startswith(SCRATCH_PREFIXES)


def _args_copy(args):
    """Host values of an Args dict: lazily read scalars resolved, arrays
    and containers copied."""
    out = {}
    for k in list(args.keys()):
        v = dict.__getitem__(args, k)
        if isinstance(v, LazyScalar):
            v = v.resolve()  # a read of one device scalar
            dict.__setitem__(args, k, v)
        if not isinstance(v, _PLAIN):
            out[k] = LIVE
        else:
            out[k] = copy.deepcopy(v) if isinstance(v, (np.ndarray, list, dict, tuple)) else v
    return out


def _objects(loop):
    return [("solver", i, s) for i, s in enumerate(loop.solvers)] + \
           [("species", i, p) for i, p in enumerate(loop.species)]


class Checkpoint:
    """The state of a run at one step (see the module docstring)."""

    def __init__(self, it, objs):
        self.it = it
        # (kind, index) -> {"dev": {...}, "args": {...}, "rng": ..., "flag_sorted": ...}
        self.objs = objs

    def nbytes(self):
        return sum(t.numel() * t.element_size() for o in self.objs.values()
                   for t in o["dev"].values())


def save_checkpoint(loop):
    """The run's state now (device tensors cloned on their stream)."""
    objs = {}
    for kind, i, obj in _objects(loop):
        dev = {k: v.clone() for k, v in obj.DataDev.items()
               if isinstance(v, torch.Tensor) and not _is_scratch(k) and k not in ALIASES}
        entry = {"dev": dev, "args": _args_copy(obj.Args)}
        rng = getattr(obj, "_rng", None)
        if rng is not None:
            entry["rng"] = copy.deepcopy(rng.bit_generator.state)
        if hasattr(obj, "flag_sorted"):
            entry["flag_sorted"] = obj.flag_sorted
        objs[(kind, i)] = entry
    return Checkpoint(loop.it, objs)


def _copy_into(pairs):
    """dst <- src for (dst, src) tensor pairs: the library's batched copy
    (32 per launch) for contiguous device tensors of whole 4-byte words,
    torch's copy for the rest."""
    dev = [(d, s_) for d, s_ in pairs if d.is_cuda and d.is_contiguous() and s_.is_contiguous()
           and (s_.numel() * s_.element_size()) % 4 == 0 and s_.numel()]
    ids = {id(d) for d, _ in dev}
    for d, s_ in pairs:
        if id(d) not in ids:
            d.copy_(s_)
    if dev:
        from ._lib import PP, call, longs, stream
        for k in range(0, len(dev), 32):
            part = dev[k:k + 32]
            call("ccl_copy_batch", len(part), longs([s_.numel() * s_.element_size()
                                                     for _, s_ in part]),
                 PP([d for d, _ in part]), PP([s_ for _, s_ in part]), stream())


def restore_checkpoint(loop, ckpt):
    """Put the run back to the checkpoint's step."""
    pairs = []
    for kind, i, obj in _objects(loop):
        entry = ckpt.objs[(kind, i)]
        # buffers that two entries name now are rebound, never written
        # through (the named aliases aside)
        ptrs = {}
        for k, t in obj.DataDev.items():
            if isinstance(t, torch.Tensor) and t.numel() and k not in ALIASES:
                ptrs.setdefault(t.data_ptr(), []).append(k)
        shared = {k for ks in ptrs.values() if len(ks) > 1 for k in ks}
        for k, v in entry["dev"].items():
            if k in ALIASES:
                continue
            cur = obj.DataDev.get(k)
            if (isinstance(cur, torch.Tensor) and k not in shared and cur.shape == v.shape
                    and cur.dtype == v.dtype and cur.device == v.device):
                pairs.append((cur, v))  # the same buffer: captured launches stay valid
            else:
                obj.DataDev[k] = v.clone()
        if hasattr(obj, "_phs_cache"):
            obj._phs_cache = {}  # phase factors: recomputed for the restored origin
        args = obj.Args
        for k in list(args.keys()):
            if k not in entry["args"]:
                del args[k]
        for k, v in entry["args"].items():
            if isinstance(v, _Live):
                continue
            dict.__setitem__(args, k, copy.deepcopy(v) if isinstance(
                v, (np.ndarray, list, dict, tuple)) else v)
        if "rng" in entry:
            obj._rng.bit_generator.state = copy.deepcopy(entry["rng"])
        if "flag_sorted" in entry:
            obj.flag_sorted = entry["flag_sorted"]
    _copy_into(pairs)
    loop.it = ckpt.it
    if hasattr(loop, "_eager_left"):
        loop._eager_left = 0  # no eager steps pending: graphs are found by signature
    # a graph whose buffers were rebound, or whose particle counts or grid
    # origin differ, fails its signature check and is captured again


def state_dict(ckpt):
    """A checkpoint in host memory (plain dicts and CPU tensors)."""
    return {"it": ckpt.it,
            "objs": {"%s:%d" % key: dict(entry, dev={k: v.cpu() for k, v in entry["dev"].items()})
                     for key, entry in ckpt.objs.items()}}


def load_state_dict(sd, device):
    """The checkpoint of a ``state_dict``, its tensors on `device`."""
    objs = {}
    for key, entry in sd["objs"].items():
        kind, i = key.split(":")
        objs[(kind, int(i))] = dict(entry, dev={k: v.to(device) for k, v in entry["dev"].items()})
    return Checkpoint(sd["it"], objs)


class Checkpointer:
    """Steps a loop and keeps a checkpoint every `every` steps (in memory):
    ``recompute(n)`` puts the run back to step n by restoring the last
    checkpoint at or before n and stepping from it."""

    def __init__(self, loop, every=10):
        if every < 1:
            raise ValueError("every must be >= 1")
        self.loop, self.every = loop, int(every)
        self.checkpoints = {}

    def step(self):
        if self.loop.it % self.every == 0 and self.loop.it not in self.checkpoints:
            self.checkpoints[self.loop.it] = save_checkpoint(self.loop)
        return self.loop.step()

    def run(self, nsteps):
        for _ in range(int(nsteps)):
            self.step()
        return self.loop.it

    def recompute(self, n):
        """The run at step n, recomputed from the last checkpoint <= n."""
        starts = [k for k in self.checkpoints if k <= n]
        if not starts:
            raise ValueError(f"no checkpoint at or before step {n}")
        restore_checkpoint(self.loop, self.checkpoints[max(starts)])
        while self.loop.it < n:
            self.loop.step()
        return self.loop.it
