"""Extract the reference's stored results into small JSON fixtures.

Run with the path of a checkout of the reference tree as its one (required)
argument; the fixtures it writes are committed, so the tests never read the
reference at run time.

  python tests/golden/make_golden.py /path/to/EDG_Westervelt

Sources (all inside the reference):
  regression.json   test/runtests.jl:207-217 (solve(3, 6, 0.1) pins, rtol 1e-9)
  convergence.json  data/convergence/results.csv (756 rows; computed with mass_solver = :cg)
  alpha_limit.json  data/alpha_limit/order.csv (difference_norms vs alpha = 0)
  steepening.json   data/steepening/{nl,lin,nl_dbc}/series.csv (all rows) and
                    recv.csv (every 32nd step), nl/snap_0.80.csv with grid.csv
                    (every 8th grid line)
"""
import csv
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _floats(path):
    with open(path) as f:
        return [[float(x) for x in row] for row in csv.reader(f) if row]


def main(ref):
    # regression pins: the two @testset "regression" blocks
    src = open(os.path.join(ref, "test", "runtests.jl")).read()
    block = src[src.index('@testset "regression"'):]
    block = block[:block.index("end\n")]
    vals = re.findall(r"e\.(erru|errv|errgradu|errE) ≈ ([0-9.eE+-]+) rtol = ([0-9.eE+-]+)", block)
    assert len(vals) == 8, vals
    pins = [dict(kw=dict(flux="upwind", mixed=True)), dict(kw=dict(flux="upwind", mixed=True, boundary="absorbing"))]
    for i, (name, v, rtol) in enumerate(vals):
        pins[i // 4][name] = float(v)
        pins[i // 4]["rtol"] = float(rtol)
    for p in pins:
        p.update(q=3, N=6, T=0.1)
    json.dump(dict(source="test/runtests.jl:207-217", cases=pins), open(os.path.join(HERE, "regression.json"), "w"),
              indent=1)

    rows = []
    with open(os.path.join(ref, "data", "convergence", "results.csv")) as f:
        for r in csv.DictReader(f):
            rows.append(dict(q=int(r["q"]), mixed=r["pairing"] == "mixed", flux=r["flux"], N=int(r["N"]),
                             erru=float(r["erru"]), errv=float(r["errv"]), errgradu=float(r["errux"]),
                             errE=float(r["errE"])))
    json.dump(dict(source="data/convergence/results.csv", T=0.1, mass_solver="cg", rows=rows),
              open(os.path.join(HERE, "convergence.json"), "w"))

    rows = []
    with open(os.path.join(ref, "data", "alpha_limit", "order.csv")) as f:
        for r in csv.DictReader(f):
            rows.append({k: float(v) for k, v in r.items()})
    json.dump(dict(source="data/alpha_limit/order.csv", q=6, N=20, T=0.5, rows=rows),
              open(os.path.join(HERE, "alpha_limit.json"), "w"), indent=1)

    st = dict(source="data/steepening", q=4, N=64, T=1.8, record_every=32, recv_stride=32, cases={})
    for case in ("nl", "lin", "nl_dbc"):
        d = os.path.join(ref, "data", "steepening", case)
        series = _floats(os.path.join(d, "series.csv"))
        recv = _floats(os.path.join(d, "recv.csv"))
        st["cases"][case] = dict(series=series, recv=[recv[i] for i in range(31, len(recv), 32)],
                                 nsteps=len(recv))
    snap = _floats(os.path.join(ref, "data", "steepening", "nl", "snap_0.80.csv"))
    grid = _floats(os.path.join(ref, "data", "steepening", "nl", "grid.csv"))
    st["snap_0.80"] = dict(stride=8, rows=[[snap[i][j] for j in range(0, len(snap[i]), 8)]
                                           for i in range(0, len(snap), 8)],
                           grid=[grid[i][0] for i in range(0, len(grid), 8)])
    json.dump(st, open(os.path.join(HERE, "steepening.json"), "w"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/EDG_Westervelt")
    main(sys.argv[1])
