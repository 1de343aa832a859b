"""The graph_mining_system binary keeps the reference's flags and log keys."""
import re
import subprocess

import pytest

from conftest import GOLDEN, PKG, pattern_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [[], ["-u"], ["-i"], ["-i", "-u", "-t", "8"]])
def test_cli_counts(sge, patterns, tmp_path, flags):
    q = tmp_path / "q.txt"
    q.write_text(pattern_of(sge, patterns, "light_query/p6").text())
    out = subprocess.run([str(PKG / "_build" / "graph_mining_system"), "-q", str(q), "-d",
                          str(GOLDEN / "ca_netscience.el"), *flags], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert re.search(r"Number of matches: 13463\b", out.stdout)
    for key in ("Planning time (s):", "use iep:", "Execution Time:", "Number of intersections:"):
        assert key in out.stdout


def test_cli_batch_and_result_file(sge, patterns, tmp_path):
    names = ["light_query/p2", "light_query/p3", "light_query/p4"]
    paths = []
    for i, n in enumerate(names):
        f = tmp_path / f"q{i}.txt"
        f.write_text(pattern_of(sge, patterns, n).text())
        paths.append(str(f))
    lst = tmp_path / "list.txt"
    lst.write_text("\n".join(paths) + "\n")
    res = tmp_path / "log.txt"
    out = subprocess.run([str(PKG / "_build" / "graph_mining_system"), "--batch", str(lst), "-d",
                          str(GOLDEN / "ca_netscience.el"), "-u", "-r", str(res)], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0
    got = [int(x) for x in re.findall(r"Number of matches: (\d+)", res.read_text())]
    assert got == [4680, 15144, 36742]


def test_cli_missing_file_exits_1(tmp_path):
    out = subprocess.run([str(PKG / "_build" / "graph_mining_system"), "-q", str(tmp_path / "nope"), "-d",
                          str(GOLDEN / "ca_netscience.el")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "Can not open file" in out.stdout


def test_cli_result_file_holds_sorted_instance_set(sge, oracle, patterns, graphs, tmp_path):
    import numpy as np
    from test_gpu_relations import sge_perms
    q = tmp_path / "q.txt"
    p = pattern_of(sge, patterns, "light_query/p4")
    q.write_text(p.text())
    res = tmp_path / "run.log"
    out = subprocess.run([str(PKG / "_build" / "graph_mining_system"), "-q", str(q), "-d",
                          str(GOLDEN / "ca_netscience.el"), "-u", "-r", str(res)], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout
    assert "Number of matches: 36742" in res.read_text()
    lines = (tmp_path / "run.log.matches").read_text().splitlines()
    assert int(lines[0]) == 36742
    got = np.array([[int(x) for x in ln.split()] for ln in lines[1:]], np.uint32)
    g = graphs("ca_netscience")
    want = oracle.canonical_instances(oracle.list_embeddings(g.offsets, g.nbrs, p.k, p.edges),
                                      np.array(sge_perms(sge, p)))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("bags", [False, True])
def test_cli_runs_the_reference_plan(sge, patterns, tmp_path, bags):
    """--plan takes the decomposition the reference printed (the first
    three-bag one it printed on ca-netscience in -u mode, inside other log
    lines) and runs it; --bags materialises its bag relations as tries.  The
    reference's count either way."""
    import json
    rows = json.loads((GOLDEN / "reference_plans.json").read_text())["rows"]
    r = next(x for x in rows if x["rc"] == 0 and x["count"] and x["mode"] == "u"
             and x["plan"].startswith("num bags: 3"))
    q = tmp_path / "q.txt"
    q.write_text(pattern_of(sge, patterns, r["pattern"]).text())
    plan = tmp_path / "plan.txt"
    plan.write_text("some log line\n" + r["plan"] + "Number of matches: (from the reference)\n")
    cmd = [str(PKG / "_build" / "graph_mining_system"), "-q", str(q), "-d", str(GOLDEN / "ca_netscience.el"), "-u",
           "--plan", str(plan)] + (["--bags"] if bags else [])
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert re.search(rf"Number of matches: {r['count']}\b", out.stdout), out.stdout
    assert "num bags: 3" in out.stdout
    assert ("bag relations:" in out.stdout) == bags


def test_cli_labeled_files(sge, oracle, graphs, tmp_path):
    """Data and query in the reference's labeled text format: the count is
    the labeled one (brute force)."""
    import numpy as np
    g = graphs("chunglu_n380")
    glab = np.random.default_rng(4).integers(0, 2, g.num_vertices).astype(np.uint32)
    d = tmp_path / "d.lg"
    g.save_labeled_text(d, glab)
    q = tmp_path / "q.lg"
    q.write_text("t 4 4\nv 0 0 2\nv 1 1 2\nv 2 0 2\nv 3 1 2\ne 0 1\ne 1 2\ne 2 3\ne 0 3\n")  # a 4-cycle, labels 0,1,0,1
    out = subprocess.run([str(PKG / "_build" / "graph_mining_system"), "-q", str(q), "-d", str(d), "-u"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    e = [(0, 1), (1, 2), (2, 3), (0, 3)]
    emb = oracle.bruteforce_embeddings_labeled(g.offsets, g.nbrs, 4, e, [0, 1, 0, 1], glab)
    inst = emb // oracle.aut_size_labeled(4, e, [0, 1, 0, 1])
    assert re.search(rf"Number of matches: {inst}\b", out.stdout), (inst, out.stdout)
