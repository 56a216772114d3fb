"""Reference-format input decks: read and write.

Abeille describes a problem in a YAML deck (src/parser.cpp:77-1054): lists
of materials, surfaces, cells and universes, the root universe, sources,
tallies, an entropy mesh and the settings.  This module reads the subset of
YAML those decks use -- block mappings and sequences, flow lists and maps
(which may span lines), plain, single- and double-quoted scalars, comments --
into plain Python values, turns a multigroup deck into a ProblemBuilder, and
writes a deck back out (floats with 17 significant digits, so a written deck
reads back bit-identical).

Entries outside the multigroup transport path (plots, cancellation, noise,
continuous-energy data) are read but not used.
"""
import math
import re

__all__ = ["parse_yaml", "load_deck", "deck_from_text", "dump_yaml"]


# ------------------------------------------------------------------ reading
def _strip_comment(line):
    out, quote = [], None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _depth(text):
    d, quote = 0, None
    for ch in text:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
    return d


def _logical_lines(text):
    """(indent, content) per logical line; flow collections left open at the
    end of a line continue on the following lines."""
    out, pending, indent = [], None, 0
    for raw in text.splitlines():
        line = _strip_comment(raw.replace("\t", "    "))
        if not line.strip():
            continue
        if pending is not None:
            pending += " " + line.strip()
            if _depth(pending) <= 0:
                out.append((indent, pending))
                pending = None
            continue
        indent = len(line) - len(line.lstrip(" "))
        content = line.strip()
        if _depth(content) > 0:
            pending = content
        else:
            out.append((indent, content))
    if pending is not None:
        raise ValueError("unterminated flow collection in deck")
    return out


_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def _scalar(tok):
    t = tok.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        return t[1:-1]
    if t in ("true", "True"):
        return True
    if t in ("false", "False"):
        return False
    if t in ("null", "~", ""):
        return None
    if _NUM.match(t):
        if re.match(r"^[+-]?\d+$", t):
            return int(t)
        return float(t)
    if t.lower() in (".inf", "+.inf"):
        return math.inf
    if t.lower() == "-.inf":
        return -math.inf
    return t


def _flow(text, i=0):
    """Parse a flow value starting at text[i]; returns (value, next index)."""
    n = len(text)
    while i < n and text[i] == " ":
        i += 1
    if i < n and text[i] == "[":
        i += 1
        out = []
        while True:
            while i < n and text[i] in " ,":
                i += 1
            if i >= n:
                raise ValueError("unterminated flow list")
            if text[i] == "]":
                return out, i + 1
            v, i = _flow(text, i)
            out.append(v)
    if i < n and text[i] == "{":
        i += 1
        out = {}
        while True:
            while i < n and text[i] in " ,":
                i += 1
            if i >= n:
                raise ValueError("unterminated flow map")
            if text[i] == "}":
                return out, i + 1
            j = i
            while j < n and text[j] != ":":
                j += 1
            key = _scalar(text[i:j])
            v, i = _flow(text, j + 1)
            out[key] = v
    # scalar up to the next , ] } at this level
    j, quote = i, None
    while j < n:
        ch = text[j]
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch in ",]}":
            break
        j += 1
    return _scalar(text[i:j]), j


def _value(text):
    text = text.strip()
    if text.startswith("[") or text.startswith("{"):
        v, _ = _flow(text)
        return v
    return _scalar(text)


def _split_key(content):
    """'key: value' -> (key, value text); None when the line is not a pair."""
    quote = None
    for i, ch in enumerate(content):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == ":" and (i + 1 == len(content) or content[i + 1] == " "):
            return _scalar(content[:i]), content[i + 1:].strip()
    return None


def _block(lines, i, indent):
    """Parse the block starting at lines[i] (indentation `indent`)."""
    if lines[i][1].startswith("- ") or lines[i][1] == "-":
        out = []
        while i < len(lines) and lines[i][0] == indent and (lines[i][1].startswith("- ") or lines[i][1] == "-"):
            rest = lines[i][1][2:].strip() if lines[i][1] != "-" else ""
            if not rest:
                i += 1
                if i < len(lines) and lines[i][0] > indent:
                    v, i = _block(lines, i, lines[i][0])
                else:
                    v = None
                out.append(v)
                continue
            kv = None if rest[0] in "[{" else _split_key(rest)
            if kv is None:
                out.append(_value(rest))
                i += 1
                continue
            # an inline mapping: its further keys sit at the column of the first
            item_indent = indent + (len(lines[i][1]) - len(rest))
            sub = [(item_indent, rest)]
            j = i + 1
            while j < len(lines) and lines[j][0] > indent:
                sub.append(lines[j])
                j += 1
            v, _ = _block(sub, 0, item_indent)
            out.append(v)
            i = j
        return out, i
    out = {}
    while i < len(lines) and lines[i][0] == indent:
        kv = _split_key(lines[i][1])
        if kv is None:
            raise ValueError(f"expected 'key: value', got {lines[i][1]!r}")
        key, rest = kv
        i += 1
        if rest:
            out[key] = _value(rest)
        elif i < len(lines) and lines[i][0] > indent:
            out[key], i = _block(lines, i, lines[i][0])
        elif i < len(lines) and lines[i][0] == indent and lines[i][1].startswith("- "):
            out[key], i = _block(lines, i, indent)  # a sequence may sit at its key's column
        else:
            out[key] = None
    return out, i


def parse_yaml(text):
    """The YAML subset of reference decks -> dict / list / scalars."""
    lines = _logical_lines(text)
    if not lines:
        return {}
    v, i = _block(lines, 0, lines[0][0])
    if i != len(lines):
        raise ValueError(f"unparsed deck content from {lines[i][1]!r}")
    return v


def deck_from_text(text, **kw):
    """ProblemBuilder for a multigroup deck given as text (see load_deck)."""
    from . import decks
    deck = parse_yaml(text)
    st = deck.get("settings", {})
    if st.get("energy-mode", "multi-group") != "multi-group":
        raise ValueError("only multigroup decks run on this engine")
    return decks.from_reference_deck(deck, **kw), deck


def load_deck(path, **kw):
    """ProblemBuilder (and the parsed deck) for the multigroup deck at `path`;
    keyword arguments (nparticles, precision, tracking) override the deck."""
    with open(path) as f:
        return deck_from_text(f.read(), **kw)


# ------------------------------------------------------------------ writing
def _fmt(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        if math.isinf(v):
            return ".inf" if v > 0 else "-.inf"
        s = "%.17g" % v
        return s if any(c in s for c in ".eEn") else s + ".0"
    if v is None:
        return "null"
    s = str(v)
    if s == "" or any(c in s for c in ":#[]{},&|~\"'") or s != s.strip() or _NUM.match(s) or s in ("true", "false"):
        return '"' + s.replace('"', '\\"') + '"'
    return s


def _flow_out(v):
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_flow_out(x) for x in v) + "]"
    if isinstance(v, dict):
        return "{" + ", ".join(f"{_fmt(k)}: {_flow_out(x)}" for k, x in v.items()) + "}"
    if hasattr(v, "tolist"):
        return _flow_out(v.tolist())
    return _fmt(v)


def dump_yaml(obj, indent=0):
    """dict / list of dicts -> deck text (lists of scalars in flow style)."""
    pad = " " * indent
    out = []
    if isinstance(obj, dict):
        for k, v in obj.items():
            if isinstance(v, dict):
                out.append(f"{pad}{_fmt(k)}:")
                out.append(dump_yaml(v, indent + 2))
            elif isinstance(v, (list, tuple)) and v and all(isinstance(x, dict) for x in v):
                out.append(f"{pad}{_fmt(k)}:")
                out.append(dump_yaml(list(v), indent + 2))
            else:
                out.append(f"{pad}{_fmt(k)}: {_flow_out(v)}")
    elif isinstance(obj, (list, tuple)):
        for item in obj:
            body = dump_yaml(item, indent + 2).splitlines()
            out.append(pad + "- " + body[0].lstrip())
            out.extend(body[1:])
    else:
        out.append(pad + _flow_out(obj))
    return "\n".join(out)
