"""Writes the one overlay header the oracle build of rsr needs.

GCC rejects the anonymous structs with SIMD members inside the unions of
src/rml/rmlv/rmlv_soa.hxx (an MSVC/clang extension).  This script reads that
header from the reference checkout and writes a variant next to the build
output in which each ``union { struct {x, y..}; struct {r, g..}; v[N]; }`` is
replaced by one union per component (``union { mvec4f x; mvec4f r; }``) and
each ``v[i]`` access by the component it aliases.  Layout and arithmetic are
unchanged.  The output lands under oracle/_ref/ (git-ignored); nothing of the
reference is stored in the repository.

usage: python make_overlay.py <reference_root> <output_root>
"""
import os
import re
import sys


def rewrite(text):
    union_re = re.compile(
        r"union\s*\{\s*((?:struct\s*\{[^}]*\};\s*|//[^\n]*\n\s*)+)mvec4f\s+v\[(\d)\];\s*\};",
        re.S)

    def fix(m):
        body, n = re.sub(r"//[^\n]*", "", m.group(1)), int(m.group(2))
        groups = [re.findall(r"\b(\w+)\b", s.replace("mvec4f", ""))
                  for s in re.findall(r"struct\s*\{([^}]*)\};", body)]
        comps = []
        for i in range(n):
            names = [g[i] for g in groups if len(g) > i]
            comps.append("union { " + " ".join("mvec4f %s;" % nm for nm in names) + " };")
        return "\n\t".join(comps)

    out = union_re.sub(fix, text)
    # v[i] -> component name (qfloat2/3/4 share x,y,z,w as the first names)
    names = ["x", "y", "z", "w"]
    out = re.sub(r"\bv\[(\d)\]", lambda m: names[int(m.group(1))], out)
    return out


def main():
    ref, dst = sys.argv[1], sys.argv[2]
    rel = os.path.join("src", "rml", "rmlv", "rmlv_soa.hxx")
    with open(os.path.join(ref, rel)) as f:
        text = f.read()
    new = rewrite(text)
    if new.count("union {") < 9:
        raise SystemExit("overlay: unexpected rmlv_soa.hxx layout")
    os.makedirs(os.path.join(dst, os.path.dirname(rel)), exist_ok=True)
    with open(os.path.join(dst, rel), "w") as f:
        f.write(new)


if __name__ == "__main__":
    main()
