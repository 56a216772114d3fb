"""Extract the reference's multigroup known-answer decks into JSON fixtures.

The reference verifies its multigroup path with analytic benchmark decks whose
expected multiplication factor is written in the deck header
(input_files/PUa-1-0-IN.yaml:2, PUb-1-0-IN.yaml:2, PUa-1-0-SL.yaml:2,
PUb-1-0-SL.yaml:2), plus decks without a stated answer used as regression
inputs (Ua-1-1-CY.yaml with P1 scattering, UD2O-2-1-SL.yaml with two groups).
This script reads those files from the reference tree (available only where the
reference is mounted), parses the small YAML subset they use, and writes
reference_decks.json next to it.  Tests read only the JSON.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = ["PUa-1-0-IN", "PUb-1-0-IN", "PUa-1-0-SL", "PUb-1-0-SL", "Ua-1-1-CY", "UD2O-2-1-SL"]


def _scalar(v):
    v = v.strip()
    if v.startswith('"') and v.endswith('"'):
        return v[1:-1]
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v)
    except ValueError:
        return v


def _flow(text):
    """Flow-style YAML ([..], {..}) -> Python, by quoting bare words and using JSON."""
    t = re.sub(r'("[^"]*")|([A-Za-z_][\w\-\.]*)', lambda m: m.group(1) or json.dumps(m.group(2)), text)
    t = re.sub(r'(?<![\w\.])(\d+)\.(?!\d)', r'\1.0', t)
    t = re.sub(r'(?<![\w"])\.(\d)', r'0.\1', t)
    return json.loads(t)


def parse_lists(path):
    # second pass: keys whose children are "- " items become lists
    text = open(path).read()
    data = {}
    cur = None
    block = []
    for raw in text.splitlines():
        s = raw.split("#", 1)[0].rstrip()
        if not s.strip():
            continue
        if not s.startswith(" ") and not s.startswith("-"):
            if cur is not None:
                data[cur] = block
            k, v = s.split(":", 1)
            if v.strip():
                data[k.strip()] = _scalar(v) if v.strip()[0] not in "[{" else _flow(v)
                cur = None
            else:
                cur = k.strip()
                block = []
        else:
            block.append(s)
    if cur is not None:
        data[cur] = block
    out = {}
    for k, v in data.items():
        if isinstance(v, list):
            out[k] = _parse_block(v)
        else:
            out[k] = v
    return out


def _parse_block(lines):
    joined, buf, depth = [], "", 0
    for s in lines:
        buf = buf + " " + s.strip() if buf else s
        depth += s.count("[") + s.count("{") - s.count("]") - s.count("}")
        if depth == 0:
            joined.append(buf)
            buf = ""
    if joined and joined[0].strip().startswith("- "):
        items, cur = [], None
        base = len(joined[0]) - len(joined[0].lstrip())
        for s in joined:
            ind = len(s) - len(s.lstrip())
            body = s.strip()
            if body.startswith("- ") and ind == base:
                item = body[2:]
                if item.startswith("{"):
                    items.append(_flow(item))
                    cur = None
                    continue
                cur = {}
                items.append(cur)
                body = item
                ind = base + 2
            k, v = body.split(":", 1)
            k, v = k.strip(), v.strip()
            if v:
                cur[k] = _flow(v) if v[0] in "[{" else _scalar(v)
            else:
                cur[k] = {}
                cur["_open"] = k
        # nested maps (sources: spatial/direction/energy)
        return _nest(items, joined, base)
    d = {}
    for s in joined:
        k, v = s.strip().split(":", 1)
        d[k.strip()] = _flow(v) if v.strip() and v.strip()[0] in "[{" else _scalar(v)
    return d


def _nest(items, joined, base):
    # rebuild with proper nesting for maps inside list items
    result, cur, sub, sub_ind = [], None, None, None
    for s in joined:
        ind = len(s) - len(s.lstrip())
        body = s.strip()
        if body.startswith("- ") and ind == base:
            item = body[2:]
            if item.startswith("{"):
                result.append(_flow(item))
                cur = None
                continue
            cur = {}
            result.append(cur)
            sub = None
            k, v = item.split(":", 1)
            if v.strip():
                cur[k.strip()] = _flow(v) if v.strip()[0] in "[{" else _scalar(v)
            else:
                sub = {}
                cur[k.strip()] = sub
                sub_ind = ind + 4
            continue
        k, v = body.split(":", 1)
        k, v = k.strip(), v.strip()
        if sub is not None and ind >= sub_ind:
            sub[k] = _flow(v) if v and v[0] in "[{" else _scalar(v)
            continue
        if v:
            cur[k] = _flow(v) if v[0] in "[{" else _scalar(v)
            sub = None
        else:
            sub = {}
            cur[k] = sub
            sub_ind = ind + 2
    return result


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = {}
    for name in DECKS:
        path = os.path.join(ref, "input_files", name + ".yaml")
        with open(path) as f:
            header = f.readline().strip() + " | " + f.readline().strip()
        m = re.search(r"k_inf\s*=\s*([0-9.]+)", header)
        deck = parse_lists(path)
        deck["_expected_k"] = float(m.group(1)) if m else None
        deck["_source"] = f"input_files/{name}.yaml"
        out[name] = deck
    with open(os.path.join(HERE, "reference_decks.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_decks.json"))


if __name__ == "__main__":
    main()
