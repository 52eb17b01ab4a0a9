"""Parameter tables of ``woo-batch`` feeding the GPU batch (``woo.batch`` counterparts).

A parametric study in the reference is a text table, one parameter set per line, and a
simulation (a script or a preprocessor); ``woo-batch`` starts one process per line with the
table and line in its options (core/main/wooMain.py:107-109, 827-852), the simulation picks its
parameters with ``readParamsFromTable`` or ``runPreprocessor`` (py/batch.py:512-631) and stores
what it found with ``writeResults`` (py/batch.py:50-164).

Here the lines of a table become scenes of one ``Batch`` (one device simulation for all lines
of a precision and step count; periodic scenes run as their own simulations): ``runTable``
builds every line's scene with the same table semantics and per-line options, runs them on the
GPU and writes one result row per line. ``TableParamReader``, ``readParamsFromTable``,
``runPreprocessor``, ``writeResults`` and ``dbReadResults`` keep the reference's names, argument
meanings and errors; text tables only (spreadsheet tables need xlrd, which is not installed) and
SQLite result files only (HDF5 needs h5py, which is not installed).
"""
import copy
import datetime
import importlib
import inspect
import json
import math
import os
import re
import runpy
import sys

import numpy as np

# increase when the layout of the results table changes (py/batch.py:27, same value)
dbFormatVersion = 3
sqliteTimeout = 1000


class _Options:
    """Batch options of the running line (wooOptions.batchTable/batchLine/batchResults of the
    reference, set there from the command line of each job; set here by ``runTable`` before it
    builds each line's scene)."""

    def __init__(self):
        self.batchTable, self.batchLine, self.batchResults = "", -1, ""


options = _Options()


def inBatch():
    """Whether a table line is being run (py/batch.py:40-43)."""
    return bool(options.batchTable)


def wait(S=None):
    """In a batch, start the line's scene ``S`` if it is not running and block until it stops
    (py/batch.py:32-38, where S is the master scene); it runs up to its stopAtStep. Does nothing
    outside a batch or without a scene."""
    if S is None or not inBatch():
        return None
    if not S.running and S.stopAtStep > S.step:
        S.run(wait=False)
    S.wait()


def _evalNamespace(**extra):
    import woodem_gb300
    ns = dict(math.__dict__)
    ns.update(woo=woodem_gb300, math=math, numpy=np, nan=float("nan"),
              Vector3=lambda x, y, z: np.array([x, y, z], float), Vector2=lambda x, y: np.array([x, y], float))
    ns.update(extra)
    return ns


class TableParamReader:
    """Simulation parameters from a text table (py/batch.py:633-837).

    * Columns are separated by blanks (no quoting); ``#`` starts a comment to the end of the line;
      lines holding nothing else are skipped (but counted).
    * The first non-empty line holds the column titles; each following non-empty line is one
      parameter set, keyed by its line number (1-based with the default ``firstLine``).
    * A value ``=`` (or an empty cell) repeats the value of the previous parameter set.
    * A column titled ``...`` (or ``…``) is appended, as text, to the column before it.
    * One trailing ``!`` is dropped from each title; a ``title`` column is synthesized when absent
      from ``name=value`` of the ``!`` columns (of all columns if none ends in ``!``), leaving out
      values ``-``, ``*`` and empty ones; a title that repeats gets ``__line=N__`` appended.
    """

    def __init__(self, file, firstLine=-1):
        if str(file).lower().endswith((".xls", ".xlsx")):
            raise NotImplementedError("%s: spreadsheet tables need the xlrd package, which is not installed; "
                                      "save the table as blank-separated text" % file)
        if firstLine < 0:
            firstLine = 0
        with open(file, "r") as f:
            raw = f.read().split("\n")
        if raw and raw[-1] == "":
            raw = raw[:-1]
        # index 0 is a placeholder so that index i is line i of the file
        text = [""] + [re.sub(r"\s*#.*", "", l) for l in raw]
        used = [i for i, l in enumerate(text) if l.strip()]
        if not used:
            raise ValueError("%s: no column titles" % file)
        headings = text[used[0]].split()
        values = {}
        for i in used[1:]:
            cells = text[i].split()
            if len(cells) < len(headings):
                raise ValueError("%s: line %d has %d columns, the titles have %d" % (file, i, len(cells), len(headings)))
            values[i + firstLine] = cells[:len(headings)]
        lines = sorted(values)
        for k, l in enumerate(lines):
            for c, v in enumerate(values[l]):
                if v in ("=", ""):
                    if k == 0:
                        raise ValueError("The = specifier on line %d, column %d, refers to nonexistent value on previous line?"
                                         % (l, c))
                    values[l][c] = values[lines[k - 1]][c]
        # continuation columns: merged into the column on their left
        kept = []
        for c, h in enumerate(headings):
            if h in ("...", "…"):
                if not kept:
                    raise ValueError("The ... header continuation is not allowed in the first column.")
                for l in lines:
                    values[l][kept[-1]] = values[l][kept[-1]] + values[l][c]
            else:
                kept.append(c)
        rawHeadings = [headings[c] for c in kept]
        for l in lines:
            values[l] = [values[l][c] for c in kept]
        names = [h[:-1] if h.endswith("!") else h for h in rawHeadings]
        self.values = {}
        for l in lines:
            self.values[l] = dict(zip(names, values[l]))
        if "title" not in names:
            hasBangs = any(h.endswith("!") for h in rawHeadings)
            seen = set()
            for l in lines:
                parts = []
                for c, h in enumerate(rawHeadings):
                    if hasBangs and not h.endswith("!"):
                        continue
                    v = values[l][c]
                    if v.strip() in ("", "-", "*"):
                        continue
                    parts.append(h.replace("!", "") + "=" + v)
                d = ",".join(parts).replace("'", "").replace('"', "")
                if d in seen:
                    d += "__line=%d__" % l
                self.values[l]["title"] = d.replace("/", "_").replace("[", "").replace("]", "").replace("*woo.unit", "")
                seen.add(d)

    def paramDict(self):
        """{line number: {column name: value as text}} with ``=`` resolved, bangs removed and the
        ``title`` column present."""
        return self.values


def parseLineList(spec, available):
    """Lines selected by ``spec`` in the ``-l/--lines`` format ``2,3-5,8`` (all of ``available``
    when ``spec`` is empty); lines absent from the table raise."""
    avail = sorted(available)
    if not spec:
        return avail
    out = []
    for part in spec.split(","):
        part = part.strip()
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-", 1)
            sel = [l for l in avail if int(a) <= l <= int(b)]
        else:
            sel = [int(part)]
        for l in sel:
            if l not in available:
                raise ValueError("line %d is not a parameter line of the table" % l)
            if l not in out:
                out.append(l)
    return out


def _tableLine():
    allTab = TableParamReader(options.batchTable).paramDict()
    if options.batchLine not in allTab:
        raise RuntimeError("Table %s doesn't contain valid line number %d" % (options.batchTable, options.batchLine))
    return allTab[options.batchLine]


def readParamsFromTable(scene, under="table", noTableOk=True, unknownOk=False, **kw):
    """Assign the parameters of the running table line to ``scene.lab.<under>`` (py/batch.py:512-580).

    ``kw`` holds every parameter with its default. Columns starting with ``!`` (job settings) and
    ``title`` are not parameters; ``*`` keeps the default, ``-`` skips the column; other values are
    evaluated as Python expressions (math functions and ``woo`` in scope). A column without a
    default raises NameError unless ``unknownOk``. Tags ``line``, ``title``, ``idt`` and ``tid`` are
    set; ``<under>.explicitParams_`` and ``<under>.defaultParams_`` list what came from the table
    and what stayed at its default."""
    S = scene
    mod = getattr(S.lab, under) if S.lab._whereIs(under) == S.labels.inMod else S.lab._newModule(under)
    tagsParams, dictParams = [], {}
    if not inBatch():
        if not noTableOk:
            raise EnvironmentError("Batch options not defined (and required; pass noTableOk=True if they are not)")
        S.tags["line"] = "l!"
    else:
        vv = dict(_tableLine())
        S.tags["line"] = "l%d" % options.batchLine
        S.tags["title"] = str(vv["title"])
        S.tags["idt"] = S.tags["id"] + "." + S.tags["title"]
        S.tags["tid"] = S.tags["title"] + "." + S.tags["id"]
        for col in vv:
            if col == "title" or col[0] == "!":
                continue
            if col not in kw and not unknownOk:
                raise NameError("Parameter `%s' has no default value assigned" % col)
            val = vv[col]
            if val == "*":
                val = kw[col]
            elif val == "-":
                continue
            elif col in kw:
                kw.pop(col)
            tagsParams.append("%s=%s" % (col, val))
            dictParams[col] = eval(val, _evalNamespace()) if isinstance(val, str) else val
    mod.defaultParams_ = ",".join("%s=%s" % (k, v) for k, v in kw.items())
    mod.explicitParams_ = ",".join(tagsParams)
    allp = dict(kw)
    allp.update(dictParams)
    for k, v in allp.items():
        setattr(mod, k, v)


def _nestedSetattr(obj, attr, val):
    parts = attr.split(".")
    for a in parts[:-1]:
        obj = getattr(obj, a)
    if not hasattr(obj, parts[-1]):
        raise AttributeError("%s: no such attribute: %s." % (type(obj).__module__ + "." + type(obj).__name__, parts[-1]))
    setattr(obj, parts[-1], val)


def runPreprocessor(pre, preFile=None):
    """Build a scene with ``pre()`` after setting the preprocessor's attributes from the running
    table line (py/batch.py:583-631). Each column except ``title`` and ``!`` columns names an
    attribute (dotted names reach nested objects); ``*``, ``-`` and empty values keep the
    preprocessor's value; values starting with ``=`` (or ``'=``) are evaluated after all others,
    with ``self`` bound to the preprocessor. Outside a batch the preprocessor runs unchanged."""
    if not inBatch():
        S = pre()
        S.tags["line"] = "default"
        S.tags["title"] = str(preFile if preFile else "[no file]")
    else:
        vv = _tableLine()
        later = []
        for name, val in vv.items():
            if name[0] == "!" or name == "title" or val in ("*", "-", ""):
                continue
            if val.startswith("="):
                later.append((name, val[1:]))
            elif val.startswith("'="):
                later.append((name, val[2:]))
            else:
                _nestedSetattr(pre, name, eval(val, _evalNamespace()))
        for name, val in later:
            _nestedSetattr(pre, name, eval(val, _evalNamespace(self=pre)))
        if hasattr(pre, "checkAttrTypes"):
            pre.checkAttrTypes()
        S = pre()
        S.tags["line"] = "l%d" % options.batchLine
        S.tags["title"] = str(vv["title"])
    S.tags["idt"] = (S.tags["id"] + "." + S.tags["title"]).replace("/", "_")
    S.tags["tid"] = (S.tags["title"] + "." + S.tags["id"]).replace("/", "_")
    return S


class _JSON(json.JSONEncoder):
    """numpy values as lists and numbers; Woo objects as {"__class__": "woo.<module>.<Class>",
    attribute: value, ...} (the form of the reference's WooJSONEncoder); anything else as text."""

    def default(self, o):
        from .core import Object
        if isinstance(o, np.ndarray):
            return o.tolist()
        if isinstance(o, np.generic):
            return o.item()
        if isinstance(o, Object):
            d = {"__class__": "woo.%s.%s" % (type(o).__module__.split(".")[-1], type(o).__name__)}
            for cls in reversed(type(o).__mro__):
                for k in getattr(cls, "_attrs", {}):
                    v = getattr(o, k, None)
                    if isinstance(v, (int, float, str, bool, list, tuple, dict, np.ndarray, np.generic, Object)) or v is None:
                        d[k] = v
            return d
        return str(o)


def _decodeObject(d):
    """The inverse of _JSON for Woo objects: an instance of the named class (woo.dem or woo.core)
    with the attributes it knows; other dicts unchanged."""
    name = d.get("__class__")
    if not isinstance(name, str) or not name.startswith("woo."):
        return d
    from . import core, dem
    cls = getattr(dem, name.split(".")[-1], None) or getattr(core, name.split(".")[-1], None)
    if cls is None:
        return d
    known = set()
    for c in cls.__mro__:
        known |= set(getattr(c, "_attrs", {}))
    return cls(**{k: v for k, v in d.items() if k in known})


_COLUMNS = ("formatVersion", "finished", "batchtable", "batchTableLine", "sceneId", "title", "duration", "pre", "tags",
            "plots", "misc", "series")


def writeResults(scene, defaultDb="woo-results.sqlite", syncXls=False, dbFmt=None, series=None, quiet=False, postHooks=[], **kw):
    """Append one row for ``scene`` to the results database (py/batch.py:50-164, SQLite layout).

    The row holds the format version, the time, the table and line (from the batch options; ''
    and -1 outside a batch), the scene's id, title, duration and tags, and ``kw`` as JSON
    (``misc``); ``series`` (a dict of 1-D sequences) as JSON. The database is the batch results
    file when in a batch, else ``defaultDb``. ``postHooks`` are called with the database name.
    ``syncXls`` would convert the database to a spreadsheet, which needs packages that are not
    installed: it raises."""
    S = scene
    if inBatch():
        table, line, db = options.batchTable, options.batchLine, options.batchResults or defaultDb
    else:
        table, line, db = "", -1, defaultDb
    if dbFmt is None:
        ext = os.path.splitext(db)[-1]
        if ext in (".sqlite", ".db"):
            dbFmt = "sqlite"
        elif ext in (".h5", ".hdf5", ".he5", ".hdf"):
            dbFmt = "hdf5"
        else:
            raise ValueError("Unable to determine database format from file extension: must be *.h5, *.hdf5, *.he5, *.hdf, "
                             "*.sqlite, *.db.")
    if dbFmt == "hdf5":
        raise NotImplementedError("HDF5 result files need h5py, which is not installed; use a *.sqlite file")
    if dbFmt != "sqlite":
        raise ValueError('*fmt* must be one of "sqlite", "hdf5", None (autodetect based on suffix)')
    if syncXls:
        raise NotImplementedError("spreadsheet export needs xlwt/openpyxl, which are not installed")
    import sqlite3
    newDb = not os.path.exists(db)
    if not quiet:
        print("Writing results to the database %s (%s)" % (db, "new" if newDb else "existing"))
    series = {} if series is None else dict(series)
    for k, v in series.items():
        if isinstance(v, np.ndarray):
            series[k] = v.tolist()
        elif not hasattr(v, "__len__"):
            raise ValueError('series["%s"] not a sequence (__len__ not defined).' % k)
    conn = sqlite3.connect(db, timeout=sqliteTimeout, detect_types=sqlite3.PARSE_DECLTYPES)
    try:
        if newDb:
            conn.execute("create table batch (formatVersion integer, finished timestamp, batchtable text, batchTableLine integer, "
                         "sceneId text, title text, duration integer, pre text, tags text, plots text, misc text, series text)")
        else:
            row = conn.execute("select formatVersion from batch").fetchone()
            if row and row[0] != dbFormatVersion:
                raise RuntimeError("database format mismatch: %s/batch/formatVersion==%s, but should be %s"
                                   % (db, row[0], dbFormatVersion))
        with conn:
            conn.execute("insert into batch values (?,?,?,?,?, ?,?,?,?,?, ?,?)",
                         (dbFormatVersion, datetime.datetime.now().isoformat(sep=" "), table, line, S.tags["id"], S.tags["title"],
                          int(getattr(S, "duration", 0)), None, json.dumps(dict(S.tags)), json.dumps({}),
                          json.dumps(kw, cls=_JSON), json.dumps(series, cls=_JSON)))
    finally:
        conn.close()
    for ph in postHooks:
        ph(db)


def dbReadResults(db, basicTypes=False):
    """Rows of a results database as dicts, oldest first (py/batch.py:172-243, SQLite): ``tags``,
    ``plots`` and ``misc`` decoded from JSON (Woo objects rebuilt), ``series`` as numpy arrays;
    with ``basicTypes`` plain JSON types throughout."""
    import sqlite3
    conn = sqlite3.connect(db, timeout=sqliteTimeout)
    conn.row_factory = sqlite3.Row
    ret = []
    try:
        for row in conn.execute("SELECT * FROM batch ORDER BY finished"):
            d = {}
            for key in row.keys():
                v = row[key]
                if key in ("pre", "tags", "plots", "misc"):
                    v = (json.loads(v) if basicTypes else json.loads(v, object_hook=_decodeObject)) if v is not None else None
                elif key == "series":
                    v = json.loads(v)
                    if not basicTypes:
                        v = {k: np.array(x) for k, x in v.items()}
                d[key] = v
            ret.append(d)
    finally:
        conn.close()
    return ret


def dbToJSON(db, **kw):
    """The results database as a JSON string (py/batch.py:245-252); ``kw`` go to json.dumps."""
    return json.dumps(dbReadResults(db, basicTypes=True), cls=_JSON, **kw)


def _flatten(obj, path="", sep=".", out=None):
    """Nested dicts and lists as {path: value}, path components joined by ``sep``."""
    if out is None:
        out = {}
    if isinstance(obj, dict):
        for k, v in obj.items():
            _flatten(v, (path + sep if path else "") + str(k), sep, out)
    elif isinstance(obj, (list, tuple)):
        for i, v in enumerate(obj):
            _flatten(v, (path + sep if path else "") + str(i), sep, out)
    else:
        out[path] = obj
    return out


def _naturalKey(s):
    return [int(t) if t.isdigit() else t for t in re.split(r"(\d+)", s)]


def dbToSpread(db, out=None, dialect="excel", rows=False, series=True, ignored=("plotData", "tags"),
               sortFirst=("title", "batchtable", "batchTableLine", "finished", "sceneId", "duration"), selector=None):
    """Flatten the rows of a results database and write them as CSV (py/batch.py:255-370): one
    column per simulation (one row with ``rows``), fields named by their path (``misc.Ek``), sorted
    naturally with ``sortFirst`` first; ``ignored`` fields and attributes left out; ``selector``
    (a function of the row dict) picks rows. Dialects ``excel`` and ``excel-tab``; spreadsheet
    files (xls, xlsx) need packages that are not installed. ``series`` are not written (they go to
    separate sheets in the reference). Writes to ``out`` or returns the text."""
    import csv
    import io
    if dialect in ("xls", "xlsx") or (out and str(out).lower().endswith((".xls", ".xlsx"))):
        raise NotImplementedError("spreadsheet output needs xlwt/openpyxl, which are not installed; use a CSV dialect")
    ign = [i.lower() for i in ignored]
    first = [f.lower() for f in sortFirst]
    recs = []
    for r in dbReadResults(db, basicTypes=True):
        if selector is not None and not selector(r):
            continue
        r = {k: v for k, v in r.items() if k.lower() not in ign and k != "series"}
        flat = _flatten(r)
        recs.append({k: v for k, v in flat.items() if k.split(".")[-1].lower() not in ign})
    fields = sorted({k for r in recs for k in r}, key=lambda f: (0, first.index(f.lower())) if f.lower() in first
                    else (1, _naturalKey(f)))
    buf = io.StringIO()
    w = csv.writer(buf, dialect=dialect)
    if rows:
        w.writerow(fields)
        for r in recs:
            w.writerow([r.get(f, "") for f in fields])
    else:
        for f in fields:
            w.writerow([f] + [r.get(f, "") for r in recs])
    text = buf.getvalue()
    if out is None:
        return text
    with open(out, "w", newline="") as fo:
        fo.write(text)


def cartProdParamTable(params, out, same=""):
    """Write a text table traversing the cartesian product of ``params`` (a dict, ordered, of
    name -> list of values; a tuple key spans several columns, its values are tuples), as
    py/batch.py:838-880 does for spreadsheets. Values equal to the line above are written as
    ``same`` ('' writes ``=``, the text form of an empty cell; None writes the value). Returns the
    number of parameter lines written."""
    import itertools
    heads, cols = [], []
    for k, vals in params.items():
        ks = list(k) if isinstance(k, tuple) else [k]
        heads.extend(ks)
        cols.append([tuple(v) if isinstance(k, tuple) else (v,) for v in vals])
    rows = [sum(combo, ()) for combo in itertools.product(*cols)]
    lines = [" ".join(heads)]
    prev = None
    for r in rows:
        cells = []
        for c, v in enumerate(r):
            s = str(v)
            if prev is not None and str(prev[c]) == s and same is not None:
                s = same if same else "="
            cells.append(s)
        if any(" " in c for c in cells):
            raise ValueError("values of a text table cannot contain blanks: %s" % cells)
        lines.append(" ".join(cells))
        prev = r
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    return len(rows)


def sceneResults(S, contacts):
    """Default result fields of a finished line: step, time, the kinetic energy of the spheres'
    nodes (translational plus rotational about the principal axes) and the number of real
    contacts."""
    from . import _plan
    A = _plan.compile_scene(S)
    nd = S.dem._nodes.soa
    sph = np.unique(A.particles["nodes"][A.particles["shape"] == 0, 0])
    m, I = nd.col("mass")[sph], nd.col("inertia")[sph]
    v, w = nd.col("vel")[sph], nd.col("angVel")[sph]
    Ek = 0.5 * float(np.sum(m * np.sum(v * v, axis=1))) + 0.5 * float(np.sum(I * w * w))
    return {"step": int(S.step), "time": float(S.time), "Ek": Ek, "nReal": int(np.count_nonzero(contacts["real"]))}


def _sceneSteps(S, steps):
    if steps is None:
        if S.stopAtStep > S.step:
            return int(S.stopAtStep - S.step)
        raise ValueError("line %s: no step count (give steps= or set Scene.stopAtStep)" % S.tags.get("line"))
    return int(steps)


def buildLine(sim, table, line, results=""):
    """The scene of one table line: ``options`` point at (table, line) while ``sim`` builds it.
    ``sim`` is a preprocessor (an object whose call returns a Scene; a copy gets the line's
    attributes through ``runPreprocessor``) or a function of no arguments that builds the scene
    itself and reads its parameters with ``readParamsFromTable``."""
    saved = (options.batchTable, options.batchLine, options.batchResults)
    options.batchTable, options.batchLine, options.batchResults = str(table), int(line), results
    try:
        if inspect.isfunction(sim) or inspect.ismethod(sim):
            S = sim()
        else:
            S = runPreprocessor(copy.deepcopy(sim))
    finally:
        options.batchTable, options.batchLine, options.batchResults = saved
    return S


def _runsAlone(S):
    """Periodic scenes, scenes whose dt changes (DynDt, Scene.nextDt) and scenes that track energy
    are not batched."""
    from .dem import DynDt
    return bool(S.isPeriodic or S.trackEnergy or any((isinstance(e, DynDt) or getattr(e, "_host", False)) and not e.dead
                                                     for e in S.engines)
                or (S.nextDt > 0 and math.isfinite(S.nextDt)))


def planTable(scenes, steps=None, max_particles=50_000_000):
    """Groups of table lines that run together: aperiodic scenes of one precision and one step
    count share a Batch, up to ``max_particles`` particles per batch; periodic scenes and scenes
    with DynDt run alone.
    ``scenes`` maps line -> Scene; returns [(kind, steps, [lines])], kind "batch" or "single"."""
    groups, order = {}, []
    out = []
    for l, S in scenes.items():
        n = _sceneSteps(S, steps)
        if _runsAlone(S):
            out.append(("single", n, [l]))
            continue
        key = (S.gpu.precision, n)
        if key not in groups:
            groups[key] = []
            order.append(key)
        groups[key].append(l)
    for key in order:
        cur, cnt = [], 0
        for l in groups[key]:
            npar = len(scenes[l].dem.par)
            if cur and cnt + npar > max_particles:
                out.append(("batch", key[1], cur))
                cur, cnt = [], 0
            cur.append(l)
            cnt += npar
        out.append(("batch", key[1], cur))
    return out


def runTable(table, sim, steps=None, lines=None, results=None, resultsFn=sceneResults, max_particles=50_000_000,
             dryRun=False, quiet=True):
    """Run the lines of a parameter table on the GPU, the lines of each group (``planTable``) as one
    Batch, and write one result row per line into ``results`` (default: the table's name with
    ``.sqlite``). ``lines`` selects lines (``-l`` format or a list). Each row's ``misc`` holds
    ``resultsFn(S, contacts)``. Returns {line: Scene}, with each scene's final node state pulled
    into its host containers (scenes run alone are closed)."""
    from .batch import Batch
    allTab = TableParamReader(table).paramDict()
    sel = parseLineList(lines, allTab) if (lines is None or isinstance(lines, str)) else list(lines)
    for l in sel:
        if l not in allTab:
            raise ValueError("line %d is not a parameter line of the table" % l)
    if results is None:
        results = os.path.splitext(str(table))[0] + ".sqlite"
    scenes = {l: buildLine(sim, table, l, results) for l in sel}
    plan = planTable(scenes, steps, max_particles)
    if dryRun:
        return plan
    for kind, n, ls in plan:
        if kind == "single":
            S = scenes[ls[0]]
            S.run(n)
            S.sync()
            found = {ls[0]: resultsFn(S, S._sim.contacts())}
            S.close()
        else:
            B = Batch([scenes[l] for l in ls])
            B.run(n)
            B.pull()
            found = {l: resultsFn(scenes[l], B.contacts(k)) for k, l in enumerate(ls)}
            B.close()
        for l in ls:
            saved = (options.batchTable, options.batchLine, options.batchResults)
            options.batchTable, options.batchLine, options.batchResults = str(table), int(l), results
            try:
                writeResults(scenes[l], defaultDb=results, quiet=quiet, **found[l])
            finally:
                options.batchTable, options.batchLine, options.batchResults = saved
    return scenes


def loadSimulation(spec):
    """The preprocessor or builder named by ``spec``: ``file.py[:name]`` (the file is run and
    ``name``, default ``pre``, taken from its globals) or ``module:name``. A class is instantiated."""
    if ":" in spec and not os.path.exists(spec):
        where, name = spec.rsplit(":", 1)
    else:
        where, name = spec, "pre"
    if where.endswith(".py"):
        obj = runpy.run_path(where)[name]
    else:
        obj = getattr(importlib.import_module(where), name)
    if inspect.isclass(obj):
        obj = obj()
    return obj


def main(argv=None):
    """``woo-batch TABLE SIMULATION`` for the GPU: every selected line of TABLE built by SIMULATION
    (``file.py[:name]`` or ``module:name``) and run, one Batch per group of lines."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m woodem_gb300.batch", description=main.__doc__)
    ap.add_argument("table")
    ap.add_argument("simulation")
    ap.add_argument("-l", "--lines", dest="lineList", default=None, help="lines of TABLE to use, e.g. 2,3-5,8 (default: all)")
    ap.add_argument("--results", dest="resultsDb", default=None, help="SQLite file for the results (default: TABLE.sqlite)")
    ap.add_argument("--steps", type=int, default=None, help="steps per line (default: each scene's stopAtStep)")
    ap.add_argument("--max-particles", type=int, default=50_000_000, help="particles per Batch")
    ap.add_argument("--dry-run", action="store_true", dest="dryRun", help="build the scenes and print the groups only")
    a = ap.parse_args(argv)
    sim = loadSimulation(a.simulation)
    out = runTable(a.table, sim, steps=a.steps, lines=a.lineList, results=a.resultsDb, max_particles=a.max_particles,
                   dryRun=a.dryRun, quiet=False)
    if a.dryRun:
        for kind, n, ls in out:
            print("%s %d steps: lines %s" % (kind, n, ",".join(str(l) for l in ls)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
