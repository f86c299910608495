"""Extract the Meng et al. spectral-upsampling tables into a C include file.

The tables are data of the paper "Physically Meaningful Rendering using
Tristimulus Colours" (Meng, Simon, Hanika, Dachsbacher 2015) as shipped in the
reference's `sub_crates/spectral_upsampling/src/meng/meng_spectra_tables.rs`
(free use confirmed by the paper's authors, see that crate's LICENSE.md).  The
values must be bit-identical to the reference's for spectral parity, so they
are parsed from that file rather than re-derived.

Usage:  python gen_spectra_tables.py <path to meng_spectra_tables.rs> [out]
Writes `spectra_tables.inc` next to this script by default.
"""
import os
import re
import sys


def _floats(text):
    return [float(x) for x in re.findall(r"-?\d+\.?\d*(?:[eE][-+]?\d+)?", text)]


def parse(src):
    out = {}
    m = re.search(r"EQUAL_ENERGY_REFLECTANCE: f32 = ([^;]+);", src)
    out["eer"] = m.group(1).strip()
    m = re.search(r"SPECTRUM_MAT_XY_TO_UV: \[f32; 6\] = \[(.*?)\];", src, re.S)
    out["xy_to_uv"] = [s.strip() for s in m.group(1).replace("\n", " ").split(",") if s.strip()]
    cells = re.findall(
        r"SpectrumGridCell \{ inside: (true|false), num_points: (\d+), idx: \[([^\]]*)\] \}", src)
    out["cells"] = [(1 if c[0] == "true" else 0, int(c[1]), [int(v) for v in c[2].split(",")])
                    for c in cells]
    pts = re.findall(
        r"SpectrumDataPoint \{\s*xystar: \(([^)]*)\),\s*uv: \(([^)]*)\),\s*spectrum: \[([^\]]*)\],?\s*\}",
        src, re.S)
    out["points"] = []
    for xy, uv, spec in pts:
        out["points"].append(([s.strip() for s in xy.split(",")], [s.strip() for s in uv.split(",")],
                              [s.strip() for s in spec.split(",") if s.strip()]))
    return out


def emit(t):
    lines = ["/* Generated by gen_spectra_tables.py from the Meng et al. spectral",
             " * upsampling tables (12x14 grid, 95 samples from 360 to 830 nm).",
             " * Do not edit. */",
             "#define PSY_MENG_GRID_WIDTH 12",
             "#define PSY_MENG_GRID_HEIGHT 14",
             "#define PSY_MENG_NUM_SAMPLES 95",
             "#define PSY_MENG_SAMPLE_MIN 360.0f",
             "#define PSY_MENG_SAMPLE_MAX 830.0f",
             "#define PSY_MENG_NUM_CELLS %d" % len(t["cells"]),
             "#define PSY_MENG_NUM_POINTS %d" % len(t["points"]),
             "#define PSY_MENG_EQUAL_ENERGY_REFLECTANCE %sf" % t["eer"],
             "PSY_MENG_CONST float psy_meng_xy_to_uv[6] = {%s};" % ", ".join(
                 v + "f" if "." in v or "e" in v else v + ".0f" for v in t["xy_to_uv"]),
             "/* inside, num_points, idx[6] */",
             "PSY_MENG_CONST int psy_meng_grid[PSY_MENG_NUM_CELLS][8] = {"]
    for inside, num, idx in t["cells"]:
        lines.append("  {%d, %d, %s}," % (inside, num, ", ".join(str(v) for v in idx)))
    lines.append("};")
    lines.append("/* uv coordinates of each data point */")
    lines.append("PSY_MENG_CONST float psy_meng_point_uv[PSY_MENG_NUM_POINTS][2] = {")

    def f(v):
        return v + "f" if ("." in v or "e" in v or "E" in v) else v + ".0f"
    for _, uv, _ in t["points"]:
        lines.append("  {%s, %s}," % (f(uv[0]), f(uv[1])))
    lines.append("};")
    lines.append("PSY_MENG_CONST float psy_meng_point_spectrum[PSY_MENG_NUM_POINTS][PSY_MENG_NUM_SAMPLES] = {")
    for _, _, spec in t["points"]:
        lines.append("  {" + ", ".join(f(v) for v in spec) + "},")
    lines.append("};")
    return "\n".join(lines) + "\n"


def main():
    src_path = sys.argv[1]
    out_path = sys.argv[2] if len(sys.argv) > 2 else os.path.join(
        os.path.dirname(os.path.abspath(__file__)), "spectra_tables.inc")
    with open(src_path) as fh:
        t = parse(fh.read())
    assert len(t["cells"]) == 168, len(t["cells"])
    assert len(t["points"]) == 186, len(t["points"])
    assert all(len(p[2]) == 95 for p in t["points"])
    with open(out_path, "w") as fh:
        fh.write(emit(t))


if __name__ == "__main__":
    main()
