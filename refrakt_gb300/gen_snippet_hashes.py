"""Writes refrakt_gb300/csrc/snippet_hashes.cpp: the snippet hash of every variation of the
reference's variations.yaml that the device code implements.

rf_compiler_create(yaml_path) accepts a caller's variations.yaml entry for evaluation only when
its src/result text hashes (snippet_hash, parsers.cpp: FNV-1a, whitespace left out) to the
reference's snippet for that name, because the kernels implement the reference's formulas and
not whatever text a file carries.  The hashes are computed by the library's own YAML reader
and hash function (parsers.cpp, compiled here with g++ into a throw-away tool), so the table
and the run-time check see the same text.

Usage: python refrakt_gb300/gen_snippet_hashes.py <reference_dir>/variations.yaml
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)

TOOL = r'''
#include <cstdio>
#include <fstream>
#include <sstream>
#include "internal.h"
namespace rfk { int fail(int status, const std::string&) { return status; } }
int main(int argc, char** argv) {
    std::ifstream f(argv[1]);
    std::stringstream ss;
    ss << f.rdbuf();
    rfk::YNode root;
    std::string err;
    if (!rfk::parse_yaml(ss.str(), root, err)) { std::fprintf(stderr, "%s\n", err.c_str()); return 1; }
    const rfk::YNode* vars = root.get("variations");
    if (!vars) return 1;
    for (const auto& [name, node] : vars->map) {
        std::string src, res;
        if (const rfk::YNode* s = node.get("src"); s && s->kind == rfk::YNode::Scalar) src = s->text;
        if (const rfk::YNode* s = node.get("result"); s && s->kind == rfk::YNode::Scalar) res = s->text;
        std::printf("%s %016llx\n", name.c_str(), (unsigned long long)rfk::snippet_hash(src, res));
    }
    return 0;
}
'''


def hashes(yaml_path):
    """name -> hash of every entry of a variations.yaml, by the library's reader."""
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "tool.cpp")
        with open(src, "w") as f:
            f.write(TOOL)
        exe = os.path.join(tmp, "tool")
        cuda = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-I", cuda,
                        src, os.path.join(CSRC, "parsers.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe, yaml_path], check=True, capture_output=True, text=True).stdout
    return dict(ln.split() for ln in out.splitlines() if ln.strip())


def main():
    sys.path.insert(0, ROOT)
    import refrakt_gb300 as R
    R.build()
    comp = R.FlameCompiler()
    h = hashes(sys.argv[1])
    rows = ["    {\"%s\", 0x%sull}," % (n, v) for n, v in sorted(h.items()) if comp.is_supported(n)]
    text = ("// GENERATED by refrakt_gb300/gen_snippet_hashes.py from the reference's variations.yaml:\n"
            "// snippet_hash (parsers.cpp) of each variation the device code implements.  A caller's\n"
            "// variations.yaml entry is evaluated only when its snippet hashes to the entry here.\n"
            "#include \"internal.h\"\n\nnamespace rfk {\n"
            "const std::map<std::string, uint64_t>& builtin_snippet_hashes() {\n"
            "    static const std::map<std::string, uint64_t> h = {\n" + "\n".join(rows) + "\n    };\n"
            "    return h;\n}\n}  // namespace rfk\n")
    with open(os.path.join(CSRC, "snippet_hashes.cpp"), "w") as f:
        f.write(text)
    print(len(rows), "snippet hashes")


if __name__ == "__main__":
    main()
