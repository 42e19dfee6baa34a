"""Regenerate the base-graph data files from the reference's tables.

The 5G NR base graphs are 3GPP TS 38.212 Tables 5.3.2-2 (BG1, 46x68) and
5.3.2-3 (BG2, 42x52).  The standard lists each nonzero entry (row i, column j)
together with its shift V_ij for the eight lifting-size sets iLS = 0..7.  The
reference stores them as sixteen dense row-major ``int[rows*cols]`` arrays, one
per (BG, iLS), with -1 for a zero block (src/h_matrices/h_bg_{1,2}_i_{0..7}.h,
selected in src/nr_ldpc.cpp:124-186).  This script reads those sixteen arrays,
checks that all eight sets share one nonzero pattern per base graph, and writes
the data back in the standard's own edge-list layout:

* ``base_graphs.inc``      -- C/CUDA arrays (compiled into the C-ABI library)
* ``../base_graphs.py``    -- the same numbers as Python data (host side, tests)

The 12x24 matrix used for the rate-1/2 Z=96 workload is the 802.11n example in
the reference's Overview.md:22-33 (the code the reference's README numbers were
measured on is no longer in its tree; this matrix is the stand-in).

Some table files write a -1 as ``- 1`` split over whitespace, so every entry is
parsed as a C expression (comma separated, whitespace removed), not by a
number regex.

Usage: python gen_base_graphs.py [reference_root]
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPES = {1: (46, 68), 2: (42, 52)}


def _parse_c_array(text, anchor):
    start = text.index("= {", text.index(anchor)) + 3
    body = text[start:text.index("}", start)]
    return [int(re.sub(r"\s+", "", tok)) for tok in body.split(",") if tok.strip()]


def load_nr_table(ref_root, bg, ils):
    path = os.path.join(ref_root, "src", "h_matrices", f"h_bg_{bg}_i_{ils}.h")
    with open(path) as f:
        vals = _parse_c_array(f.read(), "int h_base")
    rows, cols = SHAPES[bg]
    if len(vals) != rows * cols:
        raise ValueError(f"{path}: {len(vals)} entries, expected {rows * cols}")
    return [vals[r * cols:(r + 1) * cols] for r in range(rows)]


def load_wifi_matrix(ref_root):
    with open(os.path.join(ref_root, "Overview.md")) as f:
        text = f.read()
    block = text[text.index("```", text.index("802.11 base matrix")) + 3:]
    block = block[:block.index("```")]
    rows = []
    for line in block.strip().splitlines():
        vals = [int(re.sub(r"\s+", "", t)) for t in line.split(",") if t.strip()]
        rows.append(vals)
    if len(rows) != 12 or any(len(r) != 24 for r in rows):
        raise ValueError("unexpected 802.11n matrix shape")
    return rows


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NRLDPC_REF_ROOT")
    if not ref_root:
        raise SystemExit("usage: gen_base_graphs.py <reference tree> (or set NRLDPC_REF_ROOT)")
    graphs = {}
    for bg in (1, 2):
        tables = [load_nr_table(ref_root, bg, ils) for ils in range(8)]
        rows, cols = SHAPES[bg]
        edges = []
        for r in range(rows):
            for c in range(cols):
                present = [t[r][c] != -1 for t in tables]
                if any(present) and not all(present):
                    raise ValueError(f"BG{bg} ({r},{c}) pattern differs across iLS")
                if present[0]:
                    edges.append((r, c, [t[r][c] for t in tables]))
        graphs[bg] = edges
    wifi = load_wifi_matrix(ref_root)
    wifi_edges = [(r, c, v) for r, row in enumerate(wifi) for c, v in enumerate(row) if v != -1]

    # ---- C include ----------------------------------------------------------------
    out = []
    out.append("/* Generated by gen_base_graphs.py -- 3GPP TS 38.212 base graphs in the")
    out.append(" * standard's edge-list layout: one entry per nonzero block, row-major")
    out.append(" * ascending (row, then column), with the shift V for iLS = 0..7. */")
    for bg in (1, 2):
        e = graphs[bg]
        out.append(f"#define NRLDPC_BG{bg}_EDGES {len(e)}")
        out.append(f"static const unsigned char kBg{bg}Row[{len(e)}] = {{"
                   + ",".join(str(r) for r, _, _ in e) + "};")
        out.append(f"static const unsigned char kBg{bg}Col[{len(e)}] = {{"
                   + ",".join(str(c) for _, c, _ in e) + "};")
        out.append(f"static const short kBg{bg}Shift[{len(e)}][8] = {{")
        for _, _, v in e:
            out.append("  {" + ",".join(str(x) for x in v) + "},")
        out.append("};")
    out.append(f"#define NRLDPC_WIFI_EDGES {len(wifi_edges)}")
    out.append(f"static const unsigned char kWifiRow[{len(wifi_edges)}] = {{"
               + ",".join(str(r) for r, _, _ in wifi_edges) + "};")
    out.append(f"static const unsigned char kWifiCol[{len(wifi_edges)}] = {{"
               + ",".join(str(c) for _, c, _ in wifi_edges) + "};")
    out.append(f"static const short kWifiShift[{len(wifi_edges)}] = {{"
               + ",".join(str(v) for _, _, v in wifi_edges) + "};")
    with open(os.path.join(HERE, "base_graphs.inc"), "w") as f:
        f.write("\n".join(out) + "\n")

    # ---- Python data ---------------------------------------------------------------
    py = ['"""Generated by csrc/gen_base_graphs.py -- 3GPP TS 38.212 base graphs.',
          "",
          "Edge lists in the standard's layout: (row, col, (V for iLS 0..7)), row-major",
          "ascending.  WIFI_12x24 is the 802.11n rate-1/2 matrix (single shift set).",
          '"""', ""]
    for bg in (1, 2):
        py.append(f"BG{bg}_SHAPE = {SHAPES[bg]}")
        py.append(f"BG{bg}_EDGES = (")
        for r, c, v in graphs[bg]:
            py.append(f"    ({r}, {c}, {tuple(v)}),")
        py.append(")")
    py.append("WIFI_SHAPE = (12, 24)")
    py.append("WIFI_EDGES = (")
    for r, c, v in wifi_edges:
        py.append(f"    ({r}, {c}, {v}),")
    py.append(")")
    with open(os.path.join(HERE, "..", "base_graphs.py"), "w") as f:
        f.write("\n".join(py) + "\n")
    print("BG1", len(graphs[1]), "BG2", len(graphs[2]), "WIFI", len(wifi_edges))


if __name__ == "__main__":
    main()
