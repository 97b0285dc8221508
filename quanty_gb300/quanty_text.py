"""Reader for the text form Quanty's ``io.put`` writes for operators and wavefunctions.

The format is the one ``LuaInterface/lua_extensions/get_put.cpp:503-640`` prints:

* ``NewOperator( NF, NB,{ {i_(l-1), ..., i_0, value}, ... }, {{"Name",...}, ...})`` where a
  term lists its ladder operators from the leftmost factor of the product to the rightmost
  (the rightmost acts first), an index printed with ``-`` is an annihilator, and ``value`` is
  ``%23.16E`` or ``re +/- I * im``.  A term with no index is the scalar term.
* ``NewWavefunction( NF, NB,{ {"0110...", value}, ... }, ...)`` with one ``0``/``1`` character
  per fermion, orbital 0 first.

Operators are returned in the layout the C ABI takes (``include/qgpu.h``): per term the
ladder string ``o[0..l-1]`` with ``o[0]`` acting first (``Core/OperatorWaveFunction.cpp:98-113``)
and bit 15 (``CrAnMask``, ``Core/StructDef.cpp:46``) set for a creation operator.
"""
import re

CREATION = 0x8000

_num = r"[-+]?\s*(?:\d+\.?\d*(?:[eE][-+]?\d+)?|inf|nan)"
_value_re = re.compile(r"^\s*(" + _num + r")\s*(?:([-+])\s*I\s*\*\s*(" + _num + r"))?\s*$")


def _parse_value(tok):
    m = _value_re.match(tok)
    if not m:
        raise ValueError("cannot parse value %r" % tok)
    re_ = float(m.group(1).replace(" ", ""))
    im = 0.0
    if m.group(2):
        im = float(m.group(3).replace(" ", ""))
        if m.group(2) == "-":
            im = -im
    return re_, im


def _header(text, kind):
    m = re.search(kind + r"\(\s*(\d+)\s*,\s*(\d+)\s*,\s*\{", text)
    if not m:
        raise ValueError("not a %s record" % kind)
    return int(m.group(1)), int(m.group(2)), m.end()


def _body(text, start):
    """Return the text of the brace block that opens just before ``start``."""
    depth = 1
    i = start
    while depth:
        c = text[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        i += 1
    return text[start:i - 1]


def parse_operator(text):
    """Parse one ``NewOperator(...)`` record into ``{"nf", "nb", "terms"}``.

    ``terms`` is a list of ``(ops, re, im)`` with ``ops`` a tuple of uint16 ladder codes,
    ``ops[0]`` acting first.
    """
    nf, nb, start = _header(text, "NewOperator")
    body = _body(text, start)
    terms = []
    for m in re.finditer(r"\{([^{}]*)\}", body):
        toks = [t for t in m.group(1).split(",")]
        toks = [t for t in toks if t.strip() != ""]
        value = _parse_value(toks[-1])
        ladders = []
        for t in toks[:-1]:
            t = t.strip()
            if t.startswith("-"):
                ladders.append(int(t[1:].strip()))
            else:
                ladders.append(int(t) | CREATION)
        ladders.reverse()
        terms.append((tuple(ladders), value[0], value[1]))
    return {"nf": nf, "nb": nb, "terms": terms}


def parse_wavefunction(text):
    """Parse one ``NewWavefunction(...)`` record into ``{"nf", "nb", "dets", "re", "im"}``
    (plus ``complex``, ``name`` and ``nbitskey`` when the record states them)."""
    nf, nb, start = _header(text, "NewWavefunction")
    body = _body(text, start)
    dets, re_, im = [], [], []
    cplx = False
    for m in re.finditer(r'\{\s*"([01 0-9A-F]*)"\s*,([^{}]*)\}', body):
        d = m.group(1).strip()
        if nb:
            raise ValueError("bosonic determinants are not supported")
        cplx |= "I" in m.group(2)
        v = _parse_value(m.group(2))
        dets.append(d[:nf])
        re_.append(v[0])
        im.append(v[1])
    out = {"nf": nf, "nb": nb, "dets": dets, "re": re_, "im": im, "complex": cplx}
    m = re.search(r'\{"Name",\s*"((?:[^"\\]|\\.)*)"\}', text)
    if m:
        out["name"] = m.group(1)
    m = re.search(r'\{"NBitsKey",\s*(\d+)\}', text)
    if m:
        out["nbitskey"] = int(m.group(1))
    return out


def format_wavefunction(wf, var=None):
    """The ``io.put`` text of a wavefunction (LuaInterface/lua_extensions/get_put.cpp:588-634):
    one ``{"0101...", value}`` line per determinant in the stored order, values ``%23.16E`` and,
    for a complex wavefunction, ``re +/- I * |im|`` on every line; then the name and NBitsKey.
    ``wf`` is a dict as returned by :func:`parse_wavefunction` (``complex``, ``name`` and
    ``nbitskey`` default to any non-zero imaginary part, "Wave Function" and 16)."""
    cplx = wf.get("complex", any(v != 0.0 for v in wf["im"]))
    lines = []
    for d, vr, vi in zip(wf["dets"], wf["re"], wf["im"]):
        val = "%23.16E" % vr
        if cplx:
            val += (" - I * " if vi < 0 else " + I * ") + "%23.16E" % abs(vi)
        lines.append('{"%s",%s}' % (d, val))
    text = "NewWavefunction( %d, %d,{\n%s},\n{{\"Name\",\"%s\"},{\"NBitsKey\",%d}})" % (
        wf["nf"], wf.get("nb", 0), ",\n".join(lines), wf.get("name", "Wave Function"), wf.get("nbitskey", 16))
    return text if var is None else "%s = %s" % (var, text)


def format_operator(op, name="O"):
    """Write an operator back in the ``io.put`` text form (inverse of :func:`parse_operator`)."""
    lines = []
    for ops, vr, vi in op["terms"]:
        idx = []
        for o in reversed(ops):
            if o & CREATION:
                idx.append("%5d" % (o & 0x7FFF))
            else:
                idx.append("-%4d" % o)
        val = "%23.16E" % vr
        if vi != 0.0:
            val += (" - I * " if vi < 0 else " + I * ") + "%23.16E" % abs(vi)
        lines.append(" {" + ",".join(idx + [val]) + " }")
    return "%s = NewOperator( %d, %d,{\n%s},\n{{\"Name\",\"%s\"}})" % (
        name, op["nf"], op.get("nb", 0), ",\n".join(lines), name)
