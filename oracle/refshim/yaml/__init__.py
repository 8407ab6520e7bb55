"""Stand-in for PyYAML's ``safe_load`` (test infrastructure only).

It understands exactly the subset that the reference's ``constants.yaml``
uses: top-level ``KEY: value`` entries whose value is a scalar (number,
quoted string, ``null``, ``true``/``false``) or a flow-style list that may
span several lines. Block-style YAML (``- item`` lists, nested mappings) is
rejected with ``NotImplementedError``.
"""
import ast
import re

_TOP = re.compile(r"^([A-Za-z_][A-Za-z0-9_\-]*)\s*:(.*)$")


def _to_python(text):
    text = text.strip()
    if not text:
        raise NotImplementedError("block-style YAML is not supported by this stand-in")
    text = re.sub(r"\bnull\b", "None", text)
    text = re.sub(r"\btrue\b", "True", text)
    text = re.sub(r"\bfalse\b", "False", text)
    return ast.literal_eval(text)


def safe_load(stream):
    text = stream.read() if hasattr(stream, "read") else str(stream)
    result = {}
    key, buf = None, []
    for raw in text.splitlines():
        line = raw.split("#", 1)[0] if not raw.lstrip().startswith(("'", '"')) else raw
        if not line.strip():
            continue
        m = _TOP.match(line)
        if m and not line.startswith((" ", "\t")):
            if key is not None:
                result[key] = _to_python(" ".join(buf))
            key, buf = m.group(1), [m.group(2)]
        else:
            if line.lstrip().startswith("- "):
                raise NotImplementedError("block-style YAML is not supported by this stand-in")
            buf.append(line)
    if key is not None:
        result[key] = _to_python(" ".join(buf))
    return result


load = safe_load
