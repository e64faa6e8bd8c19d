"""Lists the names the reference's Python module binds (python/main.cpp): submodules, classes per
submodule and the members bound on the classes, into api_names.json (tests/test_api_surface.py).

Run from the repository root:  python tests/golden/make_api_names.py <reference-root>
"""

import json
import pathlib
import re
import sys


def _split_top(body):
    """Split a call's argument text at its top-level commas."""
    parts, depth, cur = [], 0, ""
    for ch in body:
        if ch in "(<{":
            depth += 1
        elif ch in ")>}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [x.strip() for x in parts]


def _literal(text):
    text = text.strip()
    if text in ("true", "false"):
        return text == "true"
    m = re.fullmatch(r"size_t\((.*)\)", text)
    if m:
        return int(float(m.group(1)))
    v = float(text)
    return int(v) if re.fullmatch(r"-?\d+", text) else v


def signatures(src):
    """py::arg names and defaults of every cls.def: methods by name, constructors by class."""
    methods, constructors = {}, {}
    cur, name = None, None
    pos = 0
    marks = []
    for m in re.finditer(r'def_submodule\("([A-Za-z0-9]+)"|py::class_<S>\s+cls\(sm,\s*"([A-Za-z_0-9]+)"\)', src):
        marks.append((m.start(), m.group(1), m.group(2)))
    for m in re.finditer(r"cls\.def\(", src):
        i, depth, j = m.end(), 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(src[j], 0)
            j += 1
        for k, sub, cl in marks:
            if k > m.start():
                break
            if sub:
                cur = sub
            if cl:
                name = f"{cur}.{cl}"
        parts = _split_top(src[i:j - 1])
        args = []
        for part in parts:
            a = re.fullmatch(r'py::arg\("([A-Za-z_0-9]+)"\)(?:\s*=\s*(.*))?', part, re.S)
            if a:
                args.append([a.group(1), None if a.group(2) is None else _literal(a.group(2))])
        if parts[0].startswith("py::init"):
            constructors[name] = args
        elif parts[0].startswith('"'):
            methods[parts[0].strip('"')] = args
    return methods, constructors


def main():
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {pathlib.Path(__file__).name} <root of the reference project>")
    ref = pathlib.Path(sys.argv[1])
    src = (ref / "python" / "main.cpp").read_text()
    classes = {}
    binders = {}
    # each class block: def_submodule("X") ... py::class_<S> cls(sm, "Name") ... mySystemNd*<...>(cls)
    cur, name = None, None
    for line in src.splitlines():
        m = re.search(r'def_submodule\("([A-Za-z0-9]+)"', line)
        if m:
            cur = m.group(1)
        m = re.search(r'py::class_<S>\s+cls\(sm,\s*"([A-Za-z_0-9]+)"\)', line)
        if m:
            name = f"{cur}.{m.group(1)}"
            classes.setdefault(cur, []).append(m.group(1))
            binders[name] = []
        m = re.search(r'\b(mySystemNd[A-Za-z]*)<py::class_<S>, S>\(cls\)', line)
        if m and name:
            binders[name].append(m.group(1))
    # the members each binder adds (the bodies of the template functions)
    binder_members = {}
    for b in re.finditer(r'void (mySystemNd[A-Za-z]*)\(Binder& cls\)\s*\{(.*?)\n\}', src, re.S):
        binder_members[b.group(1)] = sorted(set(re.findall(r'cls\.def(?:_property(?:_readonly)?)?\(\s*"([A-Za-z_0-9]+)"',
                                                           b.group(2))))
    members = sorted(set(re.findall(r'cls\.def(?:_property(?:_readonly)?)?\(\s*"([A-Za-z_0-9]+)"', src)) -
                     {"__repr__"})
    methods, constructors = signatures(src)
    out = pathlib.Path(__file__).parent / "api_names.json"
    out.write_text(json.dumps({"classes": classes, "members": members, "binders": binders,
                               "binder_members": binder_members, "methods": methods,
                               "constructors": constructors}, indent=1, sort_keys=True) + "\n")
    print(out, sum(len(v) for v in classes.values()), "classes", len(members), "members")


if __name__ == "__main__":
    main()
