"""Saving and loading single Woo objects (Object.dump/dumps/load/loads, lib/object/ObjectIO.hpp:28-90,
py/_monkey/io.py): ``pickle`` (any object; gzip-compressed for names ending in .gz), ``json`` and
``expr`` (a Python expression ``woo.dem.Leapfrog(damping=0.2, ...)``) for objects whose attributes
are numbers, strings, sequences or other such objects, and ``html`` (writing only). The format
is detected from the file name when writing and from the content when reading. The reference's
boost::serialization formats (xml, bin) are written here as pickles.
"""
import gzip
import json
import math
import pickle

import numpy as np

FORMATS = ("auto", "pickle", "json", "expr", "html")
_SKIP = ("field",)  # back-references to the field an engine runs on


def _className(o):
    return "woo.%s.%s" % (type(o).__module__.split(".")[-1], type(o).__name__)


def _attrs(o):
    from .core import Object
    out = {}
    for cls in reversed(type(o).__mro__):
        for k in getattr(cls, "_attrs", {}):
            if k in _SKIP:
                continue
            out[k] = getattr(o, k, None)
    for k, v in getattr(o, "__dict__", {}).items():  # list-valued attributes set by constructors
        if not k.startswith("_") and k not in out and k not in _SKIP and isinstance(v, (list, Object)):
            out[k] = v
    return out


def _plain(v, where):
    """JSON form of an attribute value."""
    from .core import Object
    if isinstance(v, Object):
        return _toJSON(v)
    if isinstance(v, (list, tuple)):
        return [_plain(x, where) for x in v]
    if isinstance(v, np.ndarray):
        return v.tolist()
    if isinstance(v, np.generic):
        return v.item()
    if isinstance(v, dict):
        return {str(k): _plain(x, where) for k, x in v.items()}
    if v is None or isinstance(v, (bool, int, float, str)):
        return v
    raise IOError("%s: attribute value of type %s cannot be written as json/expr; use the pickle format"
                  % (where, type(v).__name__))


def _toJSON(o):
    d = {"__class__": _className(o)}
    for k, v in _attrs(o).items():
        d[k] = _plain(v, "%s.%s" % (_className(o), k))
    return d


def _classByName(name):
    from . import core, dem
    if not isinstance(name, str) or not name.startswith("woo."):
        return None
    short = name.split(".")[-1]
    return getattr(dem, short, None) or getattr(core, short, None)


def _fromJSON(d):
    if isinstance(d, dict):
        cls = _classByName(d.get("__class__"))
        vals = {k: _fromJSON(v) for k, v in d.items() if k != "__class__"}
        if cls is None:
            return vals
        o = cls.__new__(cls)
        cls.__init__(o)
        for k, v in vals.items():
            setattr(o, k, v)
        return o
    if isinstance(d, list):
        return [_fromJSON(x) for x in d]
    return d


def _expr(v):
    from .core import Object
    if isinstance(v, Object):
        return "%s(%s)" % (_className(v), ", ".join("%s=%s" % (k, _expr(x)) for k, x in _attrs(v).items()))
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_expr(x) for x in v) + "]"
    if isinstance(v, np.ndarray):
        return "array(%s)" % _expr(v.tolist())
    if isinstance(v, np.generic):
        return _expr(v.item())
    if isinstance(v, float):
        if math.isnan(v):
            return "nan"
        if math.isinf(v):
            return "inf" if v > 0 else "-inf"
        return repr(v)
    if isinstance(v, dict):
        return "{" + ", ".join("%r: %s" % (str(k), _expr(x)) for k, x in v.items()) + "}"
    if v is None or isinstance(v, (bool, int, str)):
        return repr(v)
    raise IOError("attribute value of type %s cannot be written as json/expr; use the pickle format" % type(v).__name__)


def _html(o):
    rows = "".join("<tr><td>%s</td><td>%s</td></tr>" % (k, v) for k, v in _attrs(o).items())
    return "<table><tr><th colspan=\"2\">%s</th></tr>%s</table>" % (_className(o), rows)


def dumps(o, format="expr"):
    """The object as text (expr, json, html) or bytes (pickle)."""
    if format not in FORMATS or format == "auto":
        raise IOError("Unknown or unsupported format '%s' (use one of expr, json, html, pickle)" % format)
    if format == "pickle":
        return pickle.dumps(o, protocol=pickle.HIGHEST_PROTOCOL)
    if format == "json":
        return json.dumps(_toJSON(o))
    if format == "html":
        return _html(o)
    return _expr(o)


def _formatOf(name):
    n = str(name).lower()
    if n.endswith(".gz"):
        n = n[:-3]
    if n.endswith(".json"):
        return "json"
    if n.endswith((".expr", ".py")):
        return "expr"
    if n.endswith((".html", ".htm")):
        return "html"
    return "pickle"


def dump(o, out, format="auto"):
    fmt = _formatOf(out) if format == "auto" else format
    data = dumps(o, format=fmt)
    if isinstance(data, str):
        data = data.encode()
    opener = gzip.open if str(out).endswith(".gz") else open
    with opener(out, "wb") as f:
        f.write(data)


def loads(data, format="auto", cls=None):
    """An object from dumps output; the format is detected when ``auto``. With ``cls``, an
    object of another type raises TypeError."""
    import woodem_gb300
    if isinstance(data, (bytes, bytearray)):
        if data[:2] == b"\x1f\x8b":
            data = gzip.decompress(data)
        if format in ("auto", "pickle") and data[:1] == b"\x80":
            o = pickle.loads(data)
            format = "pickle"
        else:
            data = data.decode()
    if format != "pickle":
        text = data.strip()
        if format == "html":
            raise IOError("the html format cannot be read")
        if format == "json" or (format == "auto" and text.startswith("{")):
            o = _fromJSON(json.loads(text))
        elif format in ("auto", "expr"):
            ns = {"woo": woodem_gb300, "nan": float("nan"), "inf": float("inf"), "array": np.array}
            o = eval(text, ns)
        else:
            raise IOError("Unknown format '%s'" % format)
    if cls is not None and not isinstance(o, cls):
        raise TypeError("The loaded object is a %s, not a %s" % (type(o).__name__, cls.__name__))
    return o


def load(inFile, format="auto", cls=None):
    with open(inFile, "rb") as f:
        return loads(f.read(), format=format, cls=cls)
