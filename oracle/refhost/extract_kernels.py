"""Test infrastructure (part of the oracle/_ref recipe): copy the reference's
single-GPU kernels, as written, out of its src/cuda_kernels.cu into one
include file under oracle/_ref, for cuda_emu.cpp to compile on the host.

Each function is located by its signature and taken up to its closing brace
(brace counting), with a #line directive so that compiler messages point at
the reference file.  Nothing is edited: the host build supplies the CUDA
built-ins the text uses (cuda_shim.h).

    python extract_kernels.py REFERENCE_SRC_DIR OUT_FILE
"""
import re
import sys

# the kernels of the reference's mono path (src/cuda_kernels.cu) and the
# device helper they call
FUNCTIONS = [
    ("bmaxlt", r"__device__\s+LOCINT\s+bmaxlt\s*\("),
    ("read_edge_count", r"__global__\s+void\s+read_edge_count\s*\("),
    ("update_bc", r"__global__\s+void\s+update_bc\s*\("),
    ("set_degree", r"__global__\s+void\s+set_degree\s*\("),
    ("scan_col_mono2", r"__global__\s+void\s+scan_col_mono2\s*\("),
    ("scan_frt_mono", r"__global__\s+void\s+scan_frt_mono\s*\("),
    ("init_delta", r"__global__\s+void\s+init_delta\s*\("),
]


def extract(text, pattern):
    m = re.search(pattern, text)
    if not m:
        raise SystemExit(f"signature not found: {pattern}")
    start = text.rfind("\n", 0, m.start()) + 1
    i = text.index("{", m.end())
    depth = 0
    while True:
        c = text[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return start, i + 1
        i += 1


# launch-shape constants the kernels and their launches use
DEFINES = ["THREADS", "ROWXTH", "ROWXTHD"]


def main():
    src_dir, out = sys.argv[1], sys.argv[2]
    path = f"{src_dir}/cuda_kernels.cu"
    text = open(path).read()
    parts = [f"/* generated from {path}: the reference's kernels, unedited */\n"]
    for name in DEFINES:
        m = re.search(rf"^#define\s+{name}\s+.*$", text, flags=re.M)
        if not m:
            raise SystemExit(f"#define {name} not found")
        parts.append(m.group(0) + "\n")
    for name, pat in FUNCTIONS:
        a, b = extract(text, pat)
        line = text.count("\n", 0, a) + 1
        parts.append(f'#line {line} "{path}"\n{text[a:b]}\n')
    open(out, "w").write("".join(parts))


if __name__ == "__main__":
    main()
