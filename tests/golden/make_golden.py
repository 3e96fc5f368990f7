"""Regenerate the golden fixtures under tests/golden/.

Run from the repository root:  python tests/golden/make_golden.py [REFERENCE_DIR]

1. vdc_sobol_tables.npz - the two Grunschloss enumeration tables exactly as
   the reference holds them (math/ldseq/vdc_sobol_matrices52.go), parsed from
   the reference source.  Needs the reference checkout (default: the
   VERMEER_REFERENCE environment variable); skipped when it is absent.
2. colour_tables.npz plus oracle/orc_colour_tables.h and
   vermeer_gb300/csrc/colour_tables.h - the spectral tables of colour/*.go
   (CIE observer bins, Smits spectra, sRGB matrix); same reference checkout.
3. quickstart_nodes.vnf - the node examples of the reference's
   docs/quickstart.rst (the literal blocks that hold a node), each prefixed
   by a comment naming its source line; same reference checkout.
4. traversal_small.npz - small triangle soups, rays with awkward directions
   (axis-parallel, zero components, through vertices and edges, finite
   tmax) and the oracle's closest-hit and any-hit answers.  This pins the
   oracle itself, so a rebuild on another machine (x86_64 or aarch64) must
   reproduce it bit for bit.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def parse_tables(ref_dir: str):
    src = open(os.path.join(ref_dir, "math", "ldseq", "vdc_sobol_matrices52.go")).read()

    def parse(name):
        i = src.index("var " + name)
        j = src.index("\n}\n", i)
        out = np.zeros((27, 52), np.uint64)
        for m, body in re.findall(r"\{ // m = (\d+)\n(.*?)\n\t\}", src[i:j], re.S):
            vals = [int(x, 16) for x in re.findall(r"0x[0-9a-fA-F]+", body)]
            out[int(m), :len(vals)] = vals
        return out

    return parse("vdcSobolMatrices"), parse("vdcSobolMatricesInv")


def parse_colour_tables(ref_dir: str):
    """CIE 1931 2-degree observer bins, the Smits basis spectra and the sRGB
    matrix as the reference holds them (colour/*.go)."""
    src = open(os.path.join(ref_dir, "colour", "cie1931_2deg.go")).read()

    def bar(name):
        i = src.index(name + ": []float32{")
        j = src.index("},", i)
        body = src[i + len(name) + 12:j]
        return np.array([float(x) for x in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", body)], np.float32)

    sm = open(os.path.join(ref_dir, "colour", "spectrum_smits9.go")).read()
    smits = {}
    for n in ("white", "cyan", "magenta", "yellow", "red", "green", "blue"):
        mm = re.search(n + r"\s*=\s*smitsSpectrum\{([^}]*)\}", sm)
        smits[n] = np.array([float(x) for x in mm.group(1).split(",")], np.float32)
    srgb = open(os.path.join(ref_dir, "colour", "space_srgb.go")).read()
    mat = np.array([float(x) for x in re.findall(r"-?\d+\.\d+", srgb)], np.float32)
    return dict(cie_x=bar("xBar"), cie_y=bar("yBar"), cie_z=bar("zBar"), srgb=mat,
                **{"smits_" + k: v for k, v in smits.items()})


def write_colour_headers(t):
    """The same data as C arrays for the oracle and for libvmr."""
    def arr(name, vals, per=6):
        rows = []
        for i in range(0, len(vals), per):
            rows.append("    " + ", ".join(repr(float(v)) + "f" for v in vals[i:i + per]) + ",")
        return f"{name}[{len(vals)}] = {{\n" + "\n".join(rows) + "\n};\n"

    body = ("// Generated by tests/golden/make_golden.py.  CIE 1931 2-degree standard\n"
            "// observer in 5 nm bins from 360 nm, the Smits (1999) RGB->spectrum basis\n"
            "// spectra in 10 bins over [380, 720) nm, and the sRGB XYZ->RGB matrix: the\n"
            "// values of colour/cie1931_2deg.go, colour/spectrum_smits9.go and\n"
            "// colour/space_srgb.go, which spectral parity requires.\n")
    decl = {"oracle": "static const float ", "csrc": "static __constant__ const float "}
    for where, path in (("oracle", os.path.join(ROOT, "oracle", "orc_colour_tables.h")),
                        ("csrc", os.path.join(ROOT, "vermeer_gb300", "csrc", "colour_tables.h"))):
        d = decl[where]
        txt = body + "#pragma once\n"
        txt += d + arr("kCieX", t["cie_x"]) + d + arr("kCieY", t["cie_y"]) + d + arr("kCieZ", t["cie_z"])
        for k in ("white", "cyan", "magenta", "yellow", "red", "green", "blue"):
            txt += d + arr("kSmits" + k.capitalize(), t["smits_" + k], per=10)
        txt += d + arr("kSrgbFromXyz", t["srgb"], per=3)
        open(path, "w").write(txt)


def quickstart_nodes(ref_dir: str) -> str:
    """The literal blocks of docs/quickstart.rst that hold a node (a name
    followed by '{'), as one file with a comment before each."""
    lines = open(os.path.join(ref_dir, "docs", "quickstart.rst")).read().split("\n")
    out, i = [], 0
    while i < len(lines):
        if lines[i].rstrip().endswith("::"):
            j = i + 1
            while j < len(lines) and not lines[j].strip():
                j += 1
            start, block = j, []
            while j < len(lines) and (not lines[j].strip() or lines[j][:1] in (" ", "\t")):
                block.append(lines[j])
                j += 1
            text = "\n".join(block).strip("\n")
            if re.match(r"\s*[A-Za-z_]\w*\s*\{", text):
                out.append(f"# docs/quickstart.rst:{start + 1}\n{text}\n")
            i = j
        else:
            i += 1
    return "\n".join(out)


def edge_rays(verts: np.ndarray, seed: int, n_random: int) -> np.ndarray:
    """Rays aimed at vertices and edge midpoints of the soup, rays with zero
    direction components, and random rays with finite tmax."""
    from vermeer_gb300 import scenes
    rng = np.random.default_rng(seed)
    tri = verts.reshape(-1, 3, 3)
    rays = []
    # through vertices and edge midpoints, from random origins
    for k in range(min(200, tri.shape[0])):
        for tgt in (tri[k, 0], tri[k, 1], 0.5 * (tri[k, 0] + tri[k, 2])):
            o = rng.uniform(-0.5, 1.5, 3).astype(np.float32)
            d = (tgt.astype(np.float64) - o)
            d /= np.linalg.norm(d)
            rays.append([*o, *d, np.inf, 0.0])
    # axis-parallel rays (two zero direction components) from vertex-aligned origins
    for k in range(min(100, tri.shape[0])):
        v = tri[k, 0]
        for axis in range(3):
            for s in (1.0, -1.0):
                o = v.copy()
                o[axis] = -0.5 if s > 0 else 1.5
                d = np.zeros(3)
                d[axis] = s
                rays.append([*o, *d, np.inf, 0.0])
    # one zero component, origin on a vertex plane
    for k in range(min(100, tri.shape[0])):
        v = tri[k, 1]
        o = np.array([v[0], rng.uniform(-0.5, 1.5), rng.uniform(-0.5, 1.5)], np.float32)
        d = np.array([0.0, rng.normal(), rng.normal()])
        d /= np.linalg.norm(d)
        rays.append([*o, *d, np.inf, 0.0])
    rnd = scenes.incoherent_rays(n_random, seed)
    rnd[:, 6] = rng.uniform(0.0, 0.3, n_random).astype(np.float32)  # finite tmax
    out = np.concatenate([np.asarray(rays, np.float32), rnd], axis=0)
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VERMEER_REFERENCE", "")
    if ref and os.path.isdir(ref):
        fwd, inv = parse_tables(ref)
        np.savez_compressed(os.path.join(HERE, "vdc_sobol_tables.npz"), fwd=fwd, inv=inv)
        ct = parse_colour_tables(ref)
        np.savez_compressed(os.path.join(HERE, "colour_tables.npz"), **ct)
        write_colour_headers(ct)
        with open(os.path.join(HERE, "quickstart_nodes.vnf"), "w") as fh:
            fh.write(quickstart_nodes(ref))
        print("wrote vdc_sobol_tables.npz, colour_tables.npz, the colour table headers and quickstart_nodes.vnf")
    else:
        print("reference checkout not given: keeping vdc_sobol_tables.npz")

    from oracle import orc
    from vermeer_gb300 import scenes
    cases = {}
    for name, n, seed, edge in (("soup64", 64, 11, 0.2), ("soup2k", 2000, 12, 0.05), ("soup8k", 8000, 13, 0.02)):
        v, ip = scenes.triangle_soup(n, seed, edge=edge)
        rays = edge_rays(v, seed, 3000)
        m = orc.Mesh(v, ip)
        ch = m.trace(rays)
        an = m.trace(rays, shadow=True)
        cases[name] = dict(verts=v, idxp=ip, rays=rays, **{f"ch_{k}": ch[k] for k in ("prim", "t", "u", "v", "w")},
                           **{f"any_{k}": an[k] for k in ("prim", "t", "u", "v", "w")})
    flat = {f"{c}__{k}": a for c, d in cases.items() for k, a in d.items()}
    np.savez_compressed(os.path.join(HERE, "traversal_small.npz"), **flat)
    print("wrote traversal_small.npz", {c: d["rays"].shape[0] for c, d in cases.items()})


if __name__ == "__main__":
    main()
