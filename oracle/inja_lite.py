"""A small renderer for the subset of the inja template language (pantor/inja 3.x) that the
reference's shader templates use — TEST INFRASTRUCTURE ONLY (oracle/ref_build.py renders
shaders/templates/xform_select.tpl.glsl and animate.tpl.glsl with it, as src/flame.cpp:334 and
src/variation_table.cpp:260 render them with inja).

Supported: text; `{{ expr }}`; `{% for x in expr %}`, `{% for k, v in expr %}` (objects iterate
their keys in order), `{% endfor %}` with loop.index (from 0), loop.is_first, loop.is_last;
`{% if expr %}`, `{% else if expr %}`, `{% else %}`, `{% endif %}`.  Expressions: dotted paths
into the JSON data (`xform.affine.0` indexes a list), `exists("name")`, `existsIn(obj, "key")`.
"""
import re

_TOKEN = re.compile(r"\{\{(.*?)\}\}|\{%(.*?)%\}", re.S)


def _tokens(text):
    pos = 0
    for m in _TOKEN.finditer(text):
        if m.start() > pos:
            yield ("text", text[pos:m.start()])
        if m.group(1) is not None:
            yield ("expr", m.group(1).strip())
        else:
            yield ("stmt", m.group(2).strip())
        pos = m.end()
    if pos < len(text):
        yield ("text", text[pos:])


def _parse(tokens, stop=()):
    """Nodes until a statement in `stop`; returns (nodes, the stopping statement or None)."""
    nodes = []
    for kind, val in tokens:
        if kind == "stmt":
            head = val.split()[0]
            if val in stop or head in stop or (head == "else" and "else" in stop):
                return nodes, val
            if head == "for":
                m = re.match(r"for\s+(\w+)(?:\s*,\s*(\w+))?\s+in\s+(.+)$", val)
                if not m:
                    raise ValueError("bad for: " + val)
                body, end = _parse(tokens, ("endfor",))
                nodes.append(("for", m.group(1), m.group(2), m.group(3).strip(), body))
            elif head == "if":
                branches = []
                cond = val[2:].strip()
                while True:
                    body, end = _parse(tokens, ("else", "endif"))
                    branches.append((cond, body))
                    if end == "endif":
                        break
                    rest = end[4:].strip()
                    cond = rest[2:].strip() if rest.startswith("if") else "true"
                nodes.append(("if", branches))
            else:
                raise ValueError("unsupported statement: " + val)
        else:
            nodes.append((kind, val))
    if stop:
        raise ValueError("unterminated block, expected %s" % (stop,))
    return nodes, None


def _lookup(path, scope):
    parts = path.split(".")
    if parts[0] not in scope:
        raise KeyError(path)
    v = scope[parts[0]]
    for p in parts[1:]:
        v = v[int(p)] if isinstance(v, list) else v[p]
    return v


def _eval(expr, scope):
    expr = expr.strip()
    if expr == "true":
        return True
    m = re.match(r'exists\(\s*"(\w+)"\s*\)$', expr)
    if m:
        return m.group(1) in scope
    m = re.match(r'existsIn\(\s*([\w.]+)\s*,\s*"(\w+)"\s*\)$', expr)
    if m:
        obj = _lookup(m.group(1), scope)
        return isinstance(obj, dict) and m.group(2) in obj
    if re.match(r"^-?\d+$", expr):
        return int(expr)
    return _lookup(expr, scope)


def _run(nodes, scope, out):
    for n in nodes:
        if n[0] == "text":
            out.append(n[1])
        elif n[0] == "expr":
            v = _eval(n[1], scope)
            out.append(str(v).lower() if isinstance(v, bool) else str(v))
        elif n[0] == "for":
            _, a, b, src, body = n
            seq = _eval(src, scope)
            items = list(seq.items()) if isinstance(seq, dict) else list(seq)
            for i, it in enumerate(items):
                inner = dict(scope)
                if b is None:
                    inner[a] = it
                else:
                    inner[a], inner[b] = it
                inner["loop"] = {"index": i, "is_first": i == 0, "is_last": i == len(items) - 1}
                _run(body, inner, out)
        elif n[0] == "if":
            for cond, body in n[1]:
                if _eval(cond, scope):
                    _run(body, scope, out)
                    break


def render(template, data):
    nodes, _ = _parse(_tokens(template))
    out = []
    _run(nodes, dict(data), out)
    return "".join(out)
