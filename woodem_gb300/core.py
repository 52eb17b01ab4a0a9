"""``woo.core`` counterparts: Scene, Cell, Engine, Field.

Mirrors the scripting surface of core/Scene.hpp:149-190, core/Cell.hpp:137-187 and
core/Engine.hpp:27-104. A Scene owns a device-side simulation (created on the
first ``run``); engines are descriptors compiled into one device plan, so the
per-step loop of core/Scene.cpp:319-389 runs entirely on the GPU.
"""
import logging
import os
import re
import socket
import threading
import time

import numpy as np

from . import _plan

NaN = float("nan")


class Object:
    """Keyword-attribute constructor convention of Woo objects (lib/object/Object.hpp:369,417)."""

    _attrs = {}

    def __init__(self, **kw):
        for cls in reversed(type(self).__mro__):
            for k, v in getattr(cls, "_attrs", {}).items():
                if k not in self.__dict__:
                    object.__setattr__(self, k, v() if callable(v) and not isinstance(v, type) else v)
        for k, v in kw.items():
            self._setattr_checked(k, v)

    def _setattr_checked(self, k, v):
        known = set()
        for cls in type(self).__mro__:
            known |= set(getattr(cls, "_attrs", {}).keys())
        if k not in known and not hasattr(type(self), k):
            raise AttributeError("%s has no attribute '%s'" % (type(self).__name__, k))
        setattr(self, k, v)

    def updateAttrs(self, d):
        for k, v in d.items():
            self._setattr_checked(k, v)

    def __repr__(self):
        return "<%s @ %x>" % (type(self).__name__, id(self))

    # Object.dump/dumps/load/loads (lib/object/ObjectIO.hpp:28-90): woodem_gb300._objio
    def dump(self, out, format="auto"):
        from . import _objio
        _objio.dump(self, out, format)

    def dumps(self, format="expr"):
        from . import _objio
        return _objio.dumps(self, format)

    @classmethod
    def load(cls, inFile, format="auto"):
        from . import _objio
        return _objio.load(inFile, format, cls)

    @classmethod
    def loads(cls, data, format="auto"):
        from . import _objio
        return _objio.loads(data, format, cls)


class Engine(Object):
    """Base engine; ``run`` is never called on the host, engines are compiled into the device plan."""

    _attrs = {"label": "", "dead": False, "field": None}

    def critDt(self):
        return float("inf")


class PeriodicEngine(Engine):
    """Activation by step count, simulation time or wall clock (core/Engine.hpp:136-151); the
    counters (nDone, stepLast, stepPrev, virtLast, virtPrev) are updated by the runs."""
    _attrs = {"stepPeriod": 1, "virtPeriod": 0.0, "realPeriod": 0.0, "stepModulo": True, "nDo": -1, "nDone": 0,
              "initRun": True, "virtLast": NaN, "realLast": NaN, "stepLast": -1, "stepPrev": -1, "virtPrev": -1.0,
              "realPrev": -1.0}
    _COUNTERS = ("nDone", "stepLast", "stepPrev", "virtLast", "virtPrev", "realLast", "realPrev")

    def _isActivated(self, stepNow, virtNow, realNow, c=None):
        """PeriodicEngine::isActivated (core/Engine.cpp:169-194) on the counters ``c`` (a dict;
        the engine's own attributes when None), which it updates."""
        own = c is None
        if own:
            c = {k: getattr(self, k) for k in self._COUNTERS}
        init = c["stepLast"] < 0
        if init:
            c["realLast"], c["virtLast"], c["stepLast"] = realNow, virtNow, stepNow
        act = False
        if (self.nDo < 0 or c["nDone"] < self.nDo) and (
                (self.virtPeriod > 0 and virtNow - c["virtLast"] >= self.virtPeriod) or
                (self.realPeriod > 0 and realNow - c["realLast"] >= self.realPeriod) or
                (self.stepPeriod > 0 and ((stepNow - c["stepLast"] >= self.stepPeriod) or
                                          (self.stepModulo and stepNow % self.stepPeriod == 0)))):
            c["realPrev"], c["realLast"] = c["realLast"], realNow
            c["virtPrev"], c["virtLast"] = c["virtLast"], virtNow
            c["stepPrev"], c["stepLast"] = c["stepLast"], stepNow
            if not (init and not self.initRun):
                c["nDone"] += 1
                act = True
        if own:
            for k, v in c.items():
                setattr(self, k, v)
        return act


class Field(Object):
    _attrs = {}


class Cell(Object):
    """Periodic cell (core/Cell.hpp:22-187). State is integrated on the host once per step
    (core/Cell.cpp:81-120) and handed to the kernels as a handful of 3x3 matrices."""

    HomoNone, HomoPos, HomoVel, HomoVel2, HomoGradV2 = 0, 1, 2, 3, 4

    def __init__(self, **kw):
        self.hSize = np.eye(3)
        self.trsf = np.eye(3)
        self._gradV = np.zeros((3, 3))
        self.nextGradV = np.zeros((3, 3))
        self.homoDeform = Cell.HomoGradV2
        self.trsfUpperTriangular = False
        for k, v in kw.items():
            setattr(self, k, v)

    def setBox(self, *size):
        if len(size) == 1:
            size = tuple(size[0])
        self.hSize = np.diag(np.array(size, dtype=float))
        self.trsf = np.eye(3)

    @property
    def gradV(self):
        return self._gradV

    @gradV.setter
    def gradV(self, v):
        raise ValueError("Cell.gradV is not directly settable, set Cell.nextGradV instead, to be applied one step later.")

    def setCurrGradV(self, v):
        self.nextGradV = np.array(v, dtype=float)
        self._gradV = np.array(v, dtype=float)

    @property
    def size(self):
        return np.linalg.norm(np.asarray(self.hSize), axis=0)

    @property
    def volume(self):
        return float(np.linalg.det(np.asarray(self.hSize)))


_TMP = {}  # scenes saved in memory (Scene.saveTmp)


class EnergyTracker:
    """Scene.energy (core/EnergyTracker.hpp:10-80): named energies. With Scene.trackEnergy the
    entries of Leapfrog and of the contact laws are computed on the device every step and copied
    here after each run; ``kinetic``/``kinTrans``/``kinRot``/``elast`` hold the last step's value,
    the others accumulate. Entries set or added from Python stay on the host, except those of
    the device, whose new values the next run starts from."""

    def __init__(self):
        self._vals = {}
        self._resettable = set()
        self._dirty = False  # device entries changed on the host since the last run

    def _device_names(self):
        from ._native import ENERGY_NAMES
        return ENERGY_NAMES

    def __len__(self):
        return len(self._vals)

    def __getitem__(self, name):
        if name not in self._vals:
            raise KeyError("Unknown energy name '%s'." % name)
        return self._vals[name]

    def __setitem__(self, name, val):
        self._vals[name] = float(val)
        if name in self._device_names():
            self._dirty = True

    def __contains__(self, name):
        return name in self._vals

    def __iter__(self):
        return iter(self.keys())

    def add(self, dE, name, reset=False):
        """Accumulate dE into ``name`` (a resettable entry with reset=True)."""
        self._vals[name] = self._vals.get(name, 0.0) + float(dE)
        if reset:
            self._resettable.add(name)
        if name in self._device_names():
            self._dirty = True

    def clear(self):
        self._vals.clear()
        self._resettable.clear()
        self._dirty = True

    def keys(self):
        return sorted(self._vals)

    def items(self):
        return [(k, self._vals[k]) for k in self.keys()]

    def total(self):
        t = 0.0
        for k in self.keys():
            t += self._vals[k]
        return t

    def relErr(self):
        """Total energy divided by the sum of absolute values."""
        sa = sum(abs(v) for v in self._vals.values())
        return self.total() / sa if sa > 0 else 0.0

    @property
    def names(self):
        return {k: i for i, k in enumerate(self.keys())}


_LOG = logging.getLogger("woo.core")
_RE_SEQ = re.compile(r"([a-zA-Z0-9_.]+)\s*\[([0-9]+)\]")
_RE_PLAIN = re.compile(r"[a-zA-Z_][.a-zA-Z0-9_]*")


class LabelMapper:
    """Scene.labels (core/LabelMapper.hpp, core/LabelMapper.cpp): named objects of a scene,
    reached as ``S.lab.name``. A label holds a Woo object (inWoo), a sequence of Woo objects
    (inWooSeq; ``None`` items allowed, ``name[i]`` labels grow it), a plain Python object (inPy)
    or is a pseudo-module (inMod, ``S.lab._newModule('a.b')``) holding dotted labels. Engines
    and functors with a ``label`` are found automatically. Overwriting a label logs a warning
    unless it was made writable (``_setWritable``)."""
    nowhere, inWoo, inWooSeq, inPy, inMod = 0, 1, 2, 3, 4

    def __init__(self, scene=None):
        self._scene = scene
        self._woo, self._wooSeq, self._py = {}, {}, {}
        self._mods, self._writables = set(), set()

    # -- classification (LabelMapper::labelType, whereIs, ensureUsedModsOk)
    @staticmethod
    def _labelType(label):
        if label.startswith("_"):
            raise NameError("LabelMapper: labels may not start with underscore (those are reserved to access the underlying "
                            "LabelMapper object itself).")
        if label.startswith(".") or ".." in label or ".[" in label:
            raise NameError("LabelMapper: label '%s' is not a valid python identifier name." % label)
        m = _RE_SEQ.fullmatch(label)
        if m:
            return m.group(1), int(m.group(2))
        if _RE_PLAIN.fullmatch(label):
            return label, None
        raise NameError("LabelMapper: label '%s' is not a valid python identifier name." % label)

    def _autoLabels(self):
        out = {}
        for e in getattr(self._scene, "_engines", []):
            if getattr(e, "label", ""):
                out[e.label] = e
            for f in getattr(e, "_functors", lambda: [])():
                if getattr(f, "label", ""):
                    out[f.label] = f
        return out

    def _whereIs(self, label):
        if label in self._woo:
            return self.inWoo
        if label in self._wooSeq:
            return self.inWooSeq
        if label in self._py:
            return self.inPy
        if label in self._mods:
            return self.inMod
        if label in self._autoLabels():
            return self.inWoo
        return self.nowhere

    def _ensureUsedModsOk(self, label):
        parts = self._labelType(label)[0].split(".")[:-1]
        for i in range(len(parts)):
            mod = ".".join(parts[:i + 1])
            where = self._whereIs(mod)
            if where == self.nowhere:
                raise NameError("Label '%s' requires non-existent pseudo-module '%s' (use LabelMapper._newModule to create it)."
                                % (label, mod))
            if where != self.inMod:
                raise NameError("Label '%s' requires pseudo-module '%s', but this name is already used by another object."
                                % (label, mod))

    def _drop(self, label):
        for d in (self._woo, self._wooSeq, self._py):
            d.pop(label, None)

    # -- setting (LabelMapper::__setitem__ and its woo / wooSeq / py cases)
    def __setitem__(self, label, o):
        self._ensureUsedModsOk(label)
        if isinstance(o, Object):
            return self._setWoo(label, o)
        if isinstance(o, (list, tuple)):
            kind = None  # None: only None items (a sequence of Woo objects), else True (Woo) / False (python)
            for x in o:
                if x is None:
                    continue
                w = isinstance(x, Object)
                if kind is not None and kind != w:
                    raise ValueError("Sequence given to LabelMapper mixes python objects and woo.Object's.")
                kind = w
            if kind is not False:
                return self._setWooSeq(label, list(o))
        self._setPy(label, o)

    def _checkNotMod(self, label):
        if self._whereIs(label) == self.inMod:
            raise NameError("Label '%s' is a pseudo-module (cannot be overwritten)." % label)

    def _setWoo(self, label, o):
        lab0, index = self._labelType(label)
        self._checkNotMod(label)
        if index is None:
            where = self._whereIs(label)
            old = self._woo.get(label, self._py.get(label, self._wooSeq.get(label)))
            if where != self.nowhere and old is not None and old is not o and label not in self._writables:
                _LOG.warning("Label '%s' overwrites %r with %r", label, old, o)
            self._drop(label)
            self._woo[label] = o
            return
        if self._whereIs(lab0) in (self.inWoo, self.inPy):
            _LOG.warning("Sequence label '%s[%d]' creates a new sequence, deleting '%s'", lab0, index, lab0)
            self._drop(lab0)
        vec = self._wooSeq.setdefault(lab0, [])
        vec.extend([None] * (index + 1 - len(vec)))
        vec[index] = o

    def _setWooSeq(self, label, oo):
        lab0, index = self._labelType(label)
        if index is not None:
            if not oo:
                return self._setPy(label, [])
            raise NameError("Subscripted label '%s' may not be assigned a sequence of %d woo.core.Objects." % (label, len(oo)))
        self._checkNotMod(label)
        where = self._whereIs(label)
        if where != self.nowhere and (label not in self._writables or where != self.inWooSeq):
            _LOG.warning("Label '%s' overwrites an existing object with a new sequence of %d woo.Object's.", label, len(oo))
        self._drop(label)
        self._wooSeq[label] = oo

    def _setPy(self, label, o):
        lab0, index = self._labelType(label)
        self._checkNotMod(label)
        if index is None:
            where = self._whereIs(label)
            if where == self.inPy and self._py[label] is not o and label not in self._writables:
                _LOG.warning("Label '%s' overwrites %r with %r", label, self._py[label], o)
            elif where in (self.inWoo, self.inWooSeq):
                _LOG.warning("Label '%s' changes type to a pure-python object", label)
            self._drop(label)
            self._py[label] = o
            return
        where = self._whereIs(lab0)
        if where in (self.inWoo, self.inWooSeq) or (where == self.inPy and not isinstance(self._py[lab0], list)):
            _LOG.warning("Sequence label '%s[%d]' overwrites '%s' with a new python list", lab0, index, lab0)
            self._drop(lab0)
        lst = self._py.setdefault(lab0, [])
        lst.extend([None] * (index + 1 - len(lst)))
        if lst[index] is not None and label not in self._writables:
            _LOG.warning("Label '%s' overwrites old item %r with %r", label, lst[index], o)
        lst[index] = o

    # -- getting and deleting
    def __getitem__(self, label):
        m = re.fullmatch(r"(.*)\[([0-9]+)\]", label)
        if m:
            return self[m.group(1)][int(m.group(2))]
        where = self._whereIs(label)
        if where == self.nowhere:
            raise AttributeError("No such label: '%s'" % label)
        if where == self.inMod:
            raise ValueError("Label '%s' is a pseudo-module and cannot be obtained directly." % label)
        if label in self._woo:
            return self._woo[label]
        if label in self._wooSeq:
            return self._wooSeq[label]
        if label in self._py:
            return self._py[label]
        return self._autoLabels()[label]

    def __delitem__(self, label):
        where = self._whereIs(label)
        if where == self.nowhere:
            raise NameError("No such label: '%s'" % label)
        if where == self.inMod:
            pre = label + "."
            for d in (self._woo, self._wooSeq, self._py):
                for k in [k for k in d if k.startswith(pre)]:
                    del d[k]
            self._mods = {m for m in self._mods if m != label and not m.startswith(pre)}
            return
        self._drop(label)

    def __contains__(self, label):
        return self._whereIs(label) != self.nowhere

    def keys(self):
        return sorted(set(self._woo) | set(self._wooSeq) | set(self._py) | set(self._autoLabels()))

    def _setWritable(self, label):
        where = self._whereIs(label)
        if where == self.inMod:
            raise ValueError("Label '%s' cannot be made writable: is a (pseudo) module." % label)
        if where == self.nowhere:
            raise NameError("No such label: '%s'" % label)
        self._writables.add(label)

    def _newModule(self, name):
        parts = name.split(".")
        for i in range(len(parts)):
            mod = ".".join(parts[:i + 1])
            where = self._whereIs(mod)
            if where == self.inMod and i < len(parts) - 1:
                continue
            if where != self.nowhere:
                raise ValueError("Label '%s' already exists." % mod)
            self._mods.add(mod)
        return _LabelProxy(self, name)

    def _dir(self, prefix):
        pre = prefix + "." if prefix else ""
        names = set()
        for k in self.keys() + sorted(self._mods):
            if k.startswith(pre):
                names.add(k[len(pre):].split(".")[0])
        return sorted(names)


class _LabelProxy:
    """``S.lab`` and its pseudo-modules: attribute access to the labels under a prefix."""

    def __init__(self, mapper, prefix=""):
        object.__setattr__(self, "_m", mapper)
        object.__setattr__(self, "_p", prefix)

    def _full(self, name):
        return self._p + "." + name if self._p else name

    def __getattr__(self, name):
        m, p = object.__getattribute__(self, "_m"), object.__getattribute__(self, "_p")
        if name.startswith("_"):
            if not p and name in ("_newModule", "_whereIs", "_setWritable"):
                return getattr(m, name)
            raise AttributeError(name)
        full = p + "." + name if p else name
        if m._whereIs(full) == m.inMod:
            return _LabelProxy(m, full)
        return m[full]

    def __setattr__(self, name, v):
        self._m[self._full(name)] = v

    def __delattr__(self, name):
        del self._m[self._full(name)]

    def __dir__(self):
        return self._m._dir(self._p)


class Scene(Object):
    """Simulation scene. ``S.run(n)`` advances n steps of the engine list on the GPU."""

    _attrs = {
        "dt": NaN, "nextDt": NaN, "dtSafety": 0.9, "step": 0, "time": 0.0, "stopAtStep": 0,
        "trackEnergy": False, "deterministic": False, "isPeriodic": False, "tags": lambda: {},
        "subStepping": False,
    }

    def __init__(self, fields=None, **kw):
        self._engines = []
        self.fields = list(fields) if fields else []
        self.cell = Cell()
        self.gpu = _plan.GpuConfig()
        self._sim = None
        self._clock0 = time.time()
        self.labels = LabelMapper(self)
        self.energy = EnergyTracker()
        super().__init__(**kw)
        self._fillDefaultTags()
        for f in self.fields:
            f.scene = self

    def _fillDefaultTags(self):
        """Tags every new scene carries (core/Scene.cpp:140-163): user@host, isoTime and id (the local
        time as YYYYMMDDTHHMMSS, id followed by 'p' and the process id), an empty title, and
        idt/tid equal to the id. Tags given to the constructor are kept."""
        iso = time.strftime("%Y%m%dT%H%M%S", time.localtime(self._clock0))
        sid = "%sp%d" % (iso, os.getpid())
        for k, v in (("user", "%s@%s" % (os.environ.get("USER", ""), socket.gethostname())), ("isoTime", iso), ("id", sid),
                     ("title", ""), ("idt", sid), ("tid", sid)):
            self.tags.setdefault(k, v)

    def expandTags(self, s):
        """``s`` with each ``{tag}`` replaced by the value of that tag; other braces stay
        (Scene.expandTags, core/Scene.cpp:174-182)."""
        if "{" not in s:
            return s
        for k, v in self.tags.items():
            s = s.replace("{" + str(k) + "}", str(v))
        return s

    @property
    def duration(self):
        """Wall-clock seconds this scene has existed (Scene.duration, core/Scene.hpp:200)."""
        return int(time.time() - self._clock0)

    # reference name for isPeriodic in python is "periodic"
    @property
    def periodic(self):
        return self.isPeriodic

    @periodic.setter
    def periodic(self, v):
        self.isPeriodic = bool(v)
        self._invalidate()

    @property
    def engines(self):
        return self._engines

    @engines.setter
    def engines(self, ee):
        self._engines = list(ee)
        for e in self._engines:
            if getattr(e, "field", None) is None and self.fields:
                e.field = self.fields[0]
        self._invalidate()

    @property
    def dem(self):
        from .dem import DemField
        for f in self.fields:
            if isinstance(f, DemField):
                return f
        raise AttributeError("Scene has no DemField")

    @property
    def lab(self):
        """The labels of Scene.labels as attributes (``S.lab.name``, ``S.lab.module.name``):
        labeled engines and functors, objects labeled from Python and the pseudo-modules of
        ``S.lab._newModule(name)`` (e.g. ``S.lab.table`` of ``woo.batch.readParamsFromTable``)."""
        return _LabelProxy(self.labels)

    def _invalidate(self):
        if self.running and threading.current_thread() is not self.__dict__["_thread"]:
            self.__dict__["_stopFlag"] = True
            self.__dict__["_thread"].join()
        with self._lock():
            if self._sim is not None:
                self._sim.close()
                self._sim = None
        # a contact container loaded with the scene belongs to its particles as they were
        self.__dict__.pop("_pendingContacts", None)

    # --- saving and loading (lib/object/ObjectIO.hpp:28-90): the scene description and state are
    # pickled (gzip-compressed for names ending in .gz), the contact container with its persistent
    # state rides along and is uploaded with the state at the next run, so that a loaded scene
    # continues as the saved one would have.
    def __getstate__(self):
        d = self.__dict__.copy()
        d["_sim"] = None
        for k in ("_runLock", "_thread", "_except", "_stopFlag"):
            d.pop(k, None)
        return d

    def _saveBytes(self):
        import pickle
        with self._lock():  # a background run pauses between its chunks
            snap = self.__dict__.get("_pendingContacts")
            if self._sim is not None:
                from . import checkpoint
                self.sync()
                snap = checkpoint.contact_snapshot(self)
            had, old = "_pendingContacts" in self.__dict__, self.__dict__.get("_pendingContacts")
            self.__dict__["_pendingContacts"] = snap
            try:
                return pickle.dumps(self, protocol=pickle.HIGHEST_PROTOCOL)
            finally:
                if had:
                    self.__dict__["_pendingContacts"] = old
                else:
                    self.__dict__.pop("_pendingContacts", None)

    @staticmethod
    def _fromBytes(b):
        import pickle
        S = pickle.loads(b)
        if S.__dict__.get("_pendingContacts") is None:
            S.__dict__.pop("_pendingContacts", None)
        for f in S.fields:
            f.scene = S
        return S

    def save(self, fileName):
        """Save the scene (Scene.save): its description, state, contacts, engines and counters."""
        b = self._saveBytes()
        if str(fileName).endswith(".gz"):
            import gzip
            with gzip.open(fileName, "wb") as f:
                f.write(b)
        else:
            with open(fileName, "wb") as f:
                f.write(b)

    @staticmethod
    def load(fileName):
        """A scene saved with Scene.save."""
        if str(fileName).endswith(".gz"):
            import gzip
            with gzip.open(fileName, "rb") as f:
                return Scene._fromBytes(f.read())
        with open(fileName, "rb") as f:
            return Scene._fromBytes(f.read())

    def saveTmp(self, name=""):
        """Save the scene in memory under ``name`` (Scene.saveTmp)."""
        _TMP[name] = self._saveBytes()

    @staticmethod
    def loadTmp(name=""):
        """The scene saved in memory under ``name``."""
        if name not in _TMP:
            raise KeyError("No memory-saved scene named '%s'" % name)
        return Scene._fromBytes(_TMP[name])

    def deepcopy(self):
        """An independent copy of the scene (state and contacts included)."""
        return Scene._fromBytes(self._saveBytes())

    def _ensure_sim(self):
        if self._sim is None or self._sim.dirty_structure:
            if self._sim is not None:
                self._sim.close()
            self._sim = _plan.Simulation(self)
            pend = self.__dict__.pop("_pendingContacts", None)
            if pend is not None:
                from . import checkpoint
                checkpoint.restore_contacts(self, pend)
        return self._sim

    # --- running (core/Scene.cpp:33-96): run(n) queues n steps on the device; run(n, wait=False)
    # issues them from a background thread in chunks, between which stop() takes effect, and
    # wait() joins it and raises the exception the run ended with. The device simulation is used
    # by one thread at a time (the scene's lock, taken per chunk, by sync, save and close).
    _BG_CHUNK = 1000

    def _lock(self):
        lk = self.__dict__.get("_runLock")
        if lk is None:
            lk = self.__dict__["_runLock"] = threading.RLock()
        return lk

    @property
    def running(self):
        """Whether a background run (``run(wait=False)``) is in progress."""
        t = self.__dict__.get("_thread")
        return t is not None and t.is_alive()

    def run(self, nSteps=None, wait=True):
        """Run nSteps steps and set stopAtStep to the step they end at (Scene.run). Without
        nSteps, run up to stopAtStep; a background run (wait=False) without either runs until
        stop(). Raises RuntimeError while a background run is in progress."""
        if self.running:
            raise RuntimeError("Scene.run: already running")
        self.__dict__["_except"] = None
        if nSteps is not None and nSteps > 0:
            self.stopAtStep = self.step + int(nSteps)
        if nSteps is None:
            if self.stopAtStep > self.step:
                nSteps = self.stopAtStep - self.step
            elif wait:
                raise ValueError("S.run() without nSteps needs stopAtStep > step")
            else:
                nSteps = -1  # until stop()
        elif nSteps <= 0:
            return
        if wait:
            with self._lock():
                self._runSteps(int(nSteps))
            return
        self.__dict__["_stopFlag"] = False
        t = threading.Thread(target=self._backgroundLoop, args=(int(nSteps),), name="woo-scene-run", daemon=True)
        self.__dict__["_thread"] = t
        t.start()

    def _backgroundLoop(self, n):
        try:
            while n != 0 and not self.__dict__.get("_stopFlag"):
                k = self._BG_CHUNK if n < 0 else min(n, self._BG_CHUNK)
                with self._lock():
                    self._runSteps(k)
                if n > 0:
                    n -= k
        except BaseException as e:  # raised again by wait()
            self.__dict__["_except"] = e

    def paused(self):
        """Context manager that holds a background run between two chunks while its block runs
        (Scene.paused, core/Scene.cpp:98-124): ``with S.paused(): ...``."""
        return self._lock()

    def stop(self):
        """Ask a background run to stop after the chunk in progress (Scene.stop); returns at once."""
        if self.running:
            self.__dict__["_stopFlag"] = True

    def wait(self):
        """Wait for a background run to end; raise the exception it ended with (Scene.wait)."""
        t = self.__dict__.get("_thread")
        if t is not None:
            t.join()
        e = self.__dict__.get("_except")
        if e is not None:
            self.__dict__["_except"] = None
            raise e

    def one(self):
        """One step (Scene.one); RuntimeError while a background run is in progress."""
        if self.running:
            raise RuntimeError("Scene.step: already running.")
        with self._lock():
            self._runSteps(1)

    def _runSteps(self, nSteps):
        sim = self._ensure_sim()
        host = [e for e in self._engines if getattr(e, "_host", False) and not e.dead]
        if not host:
            sim.run(int(nSteps))
            return
        # engines that run on the host (VtkExport) after the device engines of a step: the queued
        # steps are cut at each step where one of them is due, then it runs on the state of that step
        left = int(nSteps)
        while left > 0:
            k = left
            now = time.time()
            for e in host:
                c = {q: getattr(e, q) for q in e._COUNTERS}
                for j in range(k):
                    if e._isActivated(self.step + j, self.time + j * self.dt, now, c):
                        k = j + 1
                        break
            step0, t0, dt0 = self.step, self.time, self.dt
            sim.run(k)
            left -= k
            due = []
            for e in host:
                for j in range(k):
                    if e._isActivated(step0 + j, t0 + j * dt0, now) and j == k - 1:
                        due.append(e)
            for e in due:
                e._runHost(self, step0 + k - 1, t0 + (k - 1) * dt0)

    def sync(self):
        """Bring device state back to the host containers."""
        with self._lock():
            if self._sim is not None:
                self._sim.pull()

    def close(self):
        """Pull the device state into the host containers and release the device simulation."""
        self._invalidate()

    def __del__(self):
        try:
            self._invalidate()
        except Exception:
            pass
