"""Regenerate the golden fixtures in this directory from the reference itself.

Needs the reference sources (REFERENCE_DIR, else $BL_REFERENCE_DIR or a
`reference` checkout beside this repository); builds them with
oracle/build_ref.sh into oracle/_ref/ and runs oracle/_ref/ref_driver, which
calls the reference's own public routines and prints full-precision results.

    python tests/golden/make_golden.py [REFERENCE_DIR]

Outputs (committed):
  <g>.mtx, <g>.initf         small seeded inputs (grid, random geometric, Chung-Lu)
  ref_<g>.npz                reference results on them:
    csr_rowptr, csr_colids   the reference reader's CSR
    L<algo>_i<iter>_{xy,f,e} layout outputs after <iter> iterations, batch 32
                             (coords, per-vertex forces of the last iteration, energy);
                             algo 2, 3, 4, 5, 6, 7, 8 at 1 and 4 iterations, algo 5
                             also at 6 (its second phase)
    conv_{xy,e,loops}        algo 2 with -engt 0.05
    bh_sorted                points after the Morton sort (BarnesHut ctor)
    bh_rep_t<theta>          BH repulsion per vertex at theta 1.2 and 0.5
    tree_*                   the reference quadtree (print_t) in canonical form
    init_greedy              initDFS coordinates
    init_rand1               randInit coordinates with one thread
  ref_stdout_grid12*.txt     stdout of the stock BatchLayout binary (format test): algo 2
                             (1 iteration), algo 5 (6 iterations), algo 7 (1 iteration)
  ref_grid64_cfg1.npz        the 64x64 triangulated grid, disc start (seed 1), algo 2,
                             batch 256, 600 iterations: the reference's final energy
                             from that start (`energy`), from five starts perturbed by
                             1e-7 relative (`ensemble`, its chaotic spread), the start
                             (`init_xy`) and the reference reader's CSR checksum

    python tests/golden/make_golden.py [REFERENCE_DIR] [--cfg1]   (--cfg1: only that file)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from batchlayoutcode_gb300 import graphs as G  # noqa: E402

BATCH = 32
ALGOS = (2, 3, 4, 5, 6, 7, 8)
ITERS = (1, 4)
EXTRA_ITERS = {5: (6,)}  # algo 5 reaches its second phase (LOOP > (int)(0.8 * 6)) at 6 iterations


def run(args, cwd=None):
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, check=True, cwd=cwd)
    if os.path.basename(args[0]) != "ref_driver":
        return r.stdout
    # the reference reader prints its progress with printf (IO.h:147-148)
    return "\n".join(l for l in r.stdout.splitlines()
                     if not l.startswith(("Converting matrix data", "Input Matrix:"))) + "\n"


def parse_block(lines, start, tag):
    head = lines[start].split()
    assert head[0] == tag, (head, tag)
    n = int(head[1])
    arr = np.array([[float(v) for v in lines[start + 1 + k].split()] for k in range(n)])
    return arr, start + 1 + n


def parse_tree(text):
    """print_tree output -> canonical node list (nodes with >= 2 children, pre-order).

    Each line is "<tabs>i:x,y:<cx>\t<cy>" for a node or "<tabs>l:x,y:<x>\t<y>"
    for a leaf point; the tab count is the depth below the root.
    """
    items = []
    for line in text.splitlines():
        if not line.strip():
            continue
        depth = len(line) - len(line.lstrip("\t"))
        body = line.strip()
        kind = body[0]
        x, y = body.split(":", 2)[2].split("\t")
        items.append((kind, depth, float(x), float(y)))
    # rebuild the tree: node -> children (by depth nesting)
    nodes = []  # dict(depth, cx, cy, children=[], leaves=count)
    stack = []
    leaf_pos = 0
    for kind, depth, x, y in items:
        while stack and nodes[stack[-1]]["depth"] >= depth:
            stack.pop()
        if kind == "i":
            nd = dict(depth=depth, cx=x, cy=y, nchild=0, lo=leaf_pos, hi=None, children=[])
            if stack:
                nodes[stack[-1]]["nchild"] += 1
                nodes[stack[-1]]["children"].append(len(nodes))
            nodes.append(nd)
            stack.append(len(nodes) - 1)
        else:
            nodes[stack[-1]]["nchild"] += 1
            leaf_pos += 1
    # second pass: a node's range ends at the leaf count when its subtree closes
    stack = []
    leaf_pos = 0
    idx = -1
    for kind, depth, x, y in items:
        while stack and nodes[stack[-1]]["depth"] >= depth:
            nodes[stack.pop()]["hi"] = leaf_pos
        if kind == "i":
            idx += 1
            stack.append(idx)
        else:
            leaf_pos += 1
    while stack:
        nodes[stack.pop()]["hi"] = leaf_pos
    keep = [nd for nd in nodes if nd["nchild"] >= 2]
    return dict(
        tree_lo=np.array([nd["lo"] for nd in keep], np.int32),
        tree_hi=np.array([nd["hi"] for nd in keep], np.int32),
        tree_depth=np.array([nd["depth"] for nd in keep], np.int32),
        tree_nchild=np.array([nd["nchild"] for nd in keep], np.int32),
        tree_centroid=np.array([[nd["cx"], nd["cy"]] for nd in keep]),
    )


def graphs():
    out = []
    g = G.grid_triangulated(12, 12)
    out.append(("grid12", g, G.init_disc(g.n, 7)))
    g = G.random_geometric(420, 6.0, seed=3)
    out.append(("rgg", g, G.init_square(g.n, 11)))
    g = G.chung_lu(400, 2.5, 8.0, seed=5)
    out.append(("chunglu", g, G.init_disc(g.n, 13)))
    return out


def config1(drv):
    """The 4,096-vertex grid workload run by the reference for 600 iterations
    of algo 2 at batch 256, from the start and from five perturbed starts."""
    g, xy = G.workload("grid64")
    xy = np.asarray(xy, np.float64)
    rng = np.random.default_rng(11)
    energies = []
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "grid64.mtx")
        G.write_mtx(g, mtx)
        lines = run([drv, "csr", mtx]).splitlines()
        rows, nnz = int(lines[0].split()[1]), int(lines[0].split()[3])
        vals = np.array([int(v) for v in lines[1:]], np.int64)
        assert np.array_equal(vals[: rows + 1], g.rowptr) and np.array_equal(vals[rows + 1: rows + 1 + nnz], g.colids)
        for k in range(6):
            start = xy if k == 0 else xy * (1.0 + 1e-7 * rng.standard_normal(xy.shape))
            initf = os.path.join(td, f"start{k}.initf")
            G.write_initf(start, initf)
            lines = run([drv, "layout", mtx, initf, "2", "600", "256", "1.2", "1.0", "0.01", td + "/"]).splitlines()
            energies.append(float(lines[0].split()[1]))
    np.savez_compressed(os.path.join(HERE, "ref_grid64_cfg1.npz"), init_xy=xy, energy=np.array(energies[0]),
                        ensemble=np.array(energies), iterations=np.array(600), batch=np.array(256),
                        csr_sum=np.array([g.n, g.nnz, int(np.sum(g.colids, dtype=np.int64))]))
    print("grid64 cfg1", energies)


def main():
    import oracle
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else oracle.reference_dir()
    if not ref:
        sys.exit("reference sources not found: pass REFERENCE_DIR or set BL_REFERENCE_DIR")
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), ref], check=True)
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    stock = os.path.join(ROOT, "oracle", "_ref", "BatchLayout")
    if "--cfg1" in sys.argv:
        config1(drv)
        return
    for name, g, xy in graphs():
        mtx = os.path.join(HERE, f"{name}.mtx")
        initf = os.path.join(HERE, f"{name}.initf")
        G.write_mtx(g, mtx)
        G.write_initf(xy, initf)
        res = {}
        lines = run([drv, "csr", mtx]).splitlines()
        rows, nnz = int(lines[0].split()[1]), int(lines[0].split()[3])
        vals = np.array([int(v) for v in lines[1:]], np.int64)
        res["csr_rowptr"] = vals[: rows + 1].astype(np.int32)
        res["csr_colids"] = vals[rows + 1: rows + 1 + nnz].astype(np.int32)
        with tempfile.TemporaryDirectory() as td:
            for algo in ALGOS:
                for it in ITERS + EXTRA_ITERS.get(algo, ()):
                    lines = run([drv, "layout", mtx, initf, str(algo), str(it), str(BATCH), "1.2", "1.0",
                                 "0.01", td + "/"]).splitlines()
                    e = float(lines[0].split()[1])
                    xy_out, k = parse_block(lines, 2, "coords")
                    f_out, _ = parse_block(lines, k, "forces")
                    res[f"L{algo}_i{it}_xy"] = xy_out
                    res[f"L{algo}_i{it}_f"] = f_out
                    res[f"L{algo}_i{it}_e"] = np.array(e)
            lines = run([drv, "layout", mtx, initf, "2", "600", str(BATCH), "1.2", "1.0", "0.05",
                         td + "/"]).splitlines()
            res["conv_e"] = np.array(float(lines[0].split()[1]))
            res["conv_loops"] = np.array(int(lines[1].split("PARAOUT")[1].split(".")[0]))
            res["conv_xy"], _ = parse_block(lines, 2, "coords")
        for theta in (1.2, 0.5):
            out = run([drv, "bh", mtx, initf, str(theta)])
            lines = out.splitlines()
            srt, k = parse_block(lines, 0, "sorted")
            rep, k = parse_block(lines, k, "repulsion")
            res[f"bh_rep_t{theta}"] = rep
            if theta == 1.2:
                res["bh_sorted"] = srt
                assert lines[k] == "tree"
                res.update(parse_tree("\n".join(lines[k + 1:])))
        lines = run([drv, "init", mtx, "0"]).splitlines()
        res["init_greedy"], _ = parse_block(lines, 0, "coords")
        lines = run([drv, "init", mtx, "1"]).splitlines()
        res["init_rand1"], _ = parse_block(lines, 0, "coords")
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **res)
        print(name, g.n, g.nnz // 2, "ok")
    # stdout layout of the stock CLI (line 18 = wall time, 19 = output path)
    for algo, iters, name in ((2, 1, "ref_stdout_grid12.txt"), (5, 6, "ref_stdout_grid12_algo5.txt"),
                              (7, 1, "ref_stdout_grid12_algo7.txt")):
        with tempfile.TemporaryDirectory() as td:
            mtx = os.path.join(HERE, "grid12.mtx")
            out = run([stock, "-input", mtx, "-output", td + "/", "-iter", str(iters), "-algo", str(algo),
                       "-threads", "1", "-initf", os.path.join(HERE, "grid12.initf"), "-batch", str(BATCH)], cwd=td)
            with open(os.path.join(HERE, name), "w") as f:
                f.write(out.replace(td + "/", "<OUTDIR>/").replace(HERE + "/", "<GOLDEN>/"))
            if algo == 2:
                with open(os.path.join(td, "grid12.mtxCACHEMINB32PARAOUT1.txt")) as fin, \
                        open(os.path.join(HERE, "ref_output_grid12.txt"), "w") as fout:
                    fout.write(fin.read())


if __name__ == "__main__":
    main()
