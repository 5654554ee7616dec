"""Minimal YAML reader for variation libraries — TEST INFRASTRUCTURE ONLY.

Covers the subset the reference's ``variations.yaml`` uses (it is read by yaml-cpp 0.6.3 in
src/variation_table.cpp:182-215): nested block mappings, ``|-`` / ``|`` literal block
scalars, single- and double-quoted scalars, ``{}`` empty maps, ``[a, b]`` flow lists,
``key:`` with a null value, and ``#`` comment lines.  PyYAML is not available here.
"""


def _strip_comment(line):
    s = line.lstrip()
    return "" if s.startswith("#") else line


def _scalar(text):
    t = text.strip()
    if not t:
        return None
    if t == "{}":
        return {}
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [x.strip() for x in inner.split(",")] if inner else []
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        body = t[1:-1]
        if t[0] == '"':
            body = body.replace('\\"', '"').replace("\\\\", "\\")
        else:
            body = body.replace("''", "'")
        return body
    return t


def parse(text):
    lines = text.split("\n")
    pos = 0

    def indent_of(s):
        return len(s) - len(s.lstrip(" "))

    def block(min_indent):
        nonlocal pos
        result = {}
        ind = None
        while pos < len(lines):
            raw = lines[pos]
            line = _strip_comment(raw)
            if not line.strip():
                pos += 1
                continue
            i = indent_of(line)
            if ind is None:
                if i < min_indent:
                    break
                ind = i
            if i < ind:
                break
            if i > ind:
                raise ValueError("unexpected indentation at line %d" % (pos + 1))
            body = line.strip()
            key, sep, rest = body.partition(":")
            if not sep:
                raise ValueError("expected key: value at line %d" % (pos + 1))
            key = key.strip()
            rest = rest.strip()
            pos += 1
            if rest in ("|-", "|"):
                collected = []
                bind = None
                while pos < len(lines):
                    raw2 = lines[pos]
                    if raw2.strip() == "":
                        collected.append("")
                        pos += 1
                        continue
                    i2 = indent_of(raw2)
                    if bind is None:
                        if i2 <= ind:
                            break
                        bind = i2
                    if i2 < bind:
                        break
                    collected.append(raw2[bind:])
                    pos += 1
                while collected and collected[-1] == "":
                    collected.pop()
                val = "\n".join(collected)
                if rest == "|":
                    val += "\n"
                result[key] = val
            elif rest == "":
                # nested mapping, or a null value
                save = pos
                while pos < len(lines) and not _strip_comment(lines[pos]).strip():
                    pos += 1
                if pos < len(lines) and indent_of(_strip_comment(lines[pos])) > ind:
                    result[key] = block(ind + 1)
                else:
                    pos = save
                    result[key] = None
            else:
                result[key] = _scalar(rest)
        return result

    return block(0)


def load(path):
    with open(path) as f:
        return parse(f.read())
