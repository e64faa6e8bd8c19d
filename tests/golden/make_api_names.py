"""Lists the names the reference's Python module binds (python/main.cpp): submodules, classes per
submodule and the members bound on the classes, into api_names.json (tests/test_api_surface.py).

Run from the repository root:  python tests/golden/make_api_names.py <reference-root>
"""

import json
import pathlib
import re
import sys


def main():
    ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
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
    out = pathlib.Path(__file__).parent / "api_names.json"
    out.write_text(json.dumps({"classes": classes, "members": members, "binders": binders,
                               "binder_members": binder_members}, indent=1, sort_keys=True) + "\n")
    print(out, sum(len(v) for v in classes.values()), "classes", len(members), "members")


if __name__ == "__main__":
    main()
