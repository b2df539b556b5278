"""Generate the golden fixtures under tests/golden/ from the reference's own
test data.  Run in a container where the pplacer sources are mounted:

    python tests/golden/make_fixtures.py /path/to/pplacer

Outputs (committed; the GPU machine never reads the reference):
  like_gtr.json, like_jtt.json, like_wag.json
      alignment, tree (post-order node arrays), model parameters and the
      PhyML tree log-likelihood that tests/pplacer/test_like.ml:71-90 expects
      (relative tolerance 1e-7, test_like.ml:30-32).  The JTT and WAG
      exchangeabilities and frequencies are read out of
      pplacer_src/prot_models.ml (lower-triangular rows, parseProtModel).
  linear_kat.json
      the masked-logdot known answers of tests/pplacer/test_linear.ml:4-28.
  gamma_kat.json
      discrete_gamma 4 0.5 from the doc comment at pplacer_src/gamma.ml:44-51.
  jplace_trees.json
      the numbered reference trees of tests/data/simple/test1.jplace and
      tests/data/trim/trim_out.jplace, with the trees parsed to post-order
      arrays (the jplace writer must reproduce the numbered strings).
  jplace_rows.json
      the placement rows of three version-3 jplace files as number tokens
      (the writer's number formatting must reproduce them).
"""
import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_fasta(path):
    names, seqs, cur = [], [], None
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            if line.startswith(">"):
                names.append(line[1:].split()[0])
                seqs.append([])
            else:
                seqs[-1].append(line)
    return names, ["".join(s).upper() for s in seqs]


def parse_newick(text):
    """Post-order numbering as pplacer_src/newick_parser.mly:50-59: each leaf
    gets the next id when read, each internal node when its ')' closes."""
    text = text.strip()
    pos = 0
    parent, bl, label = [], [], []

    def new_node(lab):
        parent.append(-1)
        bl.append(0.0)
        label.append(lab)
        return len(parent) - 1

    def read_label():
        nonlocal pos
        start = pos
        while pos < len(text) and text[pos] not in ",():;[":
            pos += 1
        return text[start:pos].strip()

    def read_bl(node):
        nonlocal pos
        if pos < len(text) and text[pos] == ":":
            pos += 1
            start = pos
            while pos < len(text) and text[pos] not in ",();[":
                pos += 1
            bl[node] = float(text[start:pos])

    def subtree():
        nonlocal pos
        if text[pos] == "(":
            pos += 1
            kids = [subtree()]
            while text[pos] == ",":
                pos += 1
                kids.append(subtree())
            assert text[pos] == ")"
            pos += 1
            lab = read_label()
            node = new_node(lab)
            for k in kids:
                parent[k] = node
        else:
            node = new_node(read_label())
        read_bl(node)
        return node

    root = subtree()
    assert parent[root] == -1
    return parent, bl, label


def ocaml_list_block(src, name):
    m = re.search(r"let %s\s*=\s*parseProtModel\s*\[\|(.*?)\|\]" % name, src, re.S)
    rows = re.findall(r'"([^"]*)"', m.group(1))
    return [[float(v) for v in r.split()] for r in rows]


def ocaml_freq(src, name):
    m = re.search(r'let %s\s*=\s*parseFreq\s*"([^"]*)"' % name, src)
    return [float(v) for v in m.group(1).split()]


def prot_exch(lower):
    n = len(lower) + 1
    m = [[0.0] * n for _ in range(n)]
    for i in range(n):
        for j in range(n):
            if i != j:
                m[i][j] = lower[max(i, j) - 1][min(i, j)]
    return m


def gtr_exch(rates):
    ac, ag, at, cg, ct, gt = rates
    return [[0, ac, ag, at], [ac, 0, cg, ct], [ag, cg, 0, gt], [at, ct, gt, 0]]


def like_fixture(ref_root, sub, fasta, tree, expected):
    d = os.path.join(ref_root, "tests", "data", "like", sub)
    names, seqs = read_fasta(os.path.join(d, fasta))
    with open(os.path.join(d, tree)) as f:
        parent, bl, label = parse_newick(f.read())
    with open(os.path.join(d, "phylo_model.jplace")) as f:
        pm = json.load(f)
    leaf_row = [names.index(l) if l else -1 for l in label]
    model = {"subs_model": pm["subs_model"], "empirical_frequencies": pm["empirical_frequencies"],
             "gamma_alpha": pm["gamma"]["alpha"], "gamma_n_cats": pm["gamma"]["n_cats"]}
    if pm["subs_model"] == "GTR":
        r = pm["subs_rates"]
        model["exch"] = gtr_exch([r[k] for k in ("ac", "ag", "at", "cg", "ct", "gt")])
        model["statd"] = None  # empirical, from the alignment
    else:
        src = open(os.path.join(ref_root, "pplacer_src", "prot_models.ml")).read()
        key = pm["subs_model"].lower()
        model["exch"] = prot_exch(ocaml_list_block(src, key + "_trans"))
        model["statd"] = ocaml_freq(src, key + "_statd")
    return {"source": "tests/data/like/%s (pplacer tests/pplacer/test_like.ml)" % sub,
            "names": names, "seqs": seqs, "parent": parent, "bl": bl, "label": label,
            "leaf_row": leaf_row, "model": model, "expected_loglike": expected, "rel_tol": 1e-7}


def main(ref_root):
    fx = {
        "gtr": like_fixture(ref_root, "gtr", "hiv.fasta", "hiv.phy_phyml_tree.txt", -1752.42340),
        "jtt": like_fixture(ref_root, "jtt", "actin.fasta", "actin.phy_phyml_tree.txt", -2326.22075),
        "wag": like_fixture(ref_root, "wag", "actin.fasta", "actin.phy_phyml_tree.txt", -2334.79151),
    }
    for k, v in fx.items():
        with open(os.path.join(HERE, "like_%s.json" % k), "w") as f:
            json.dump(v, f, indent=0)
    # tests/pplacer/test_linear.ml:4-28
    kat = {
        "mask": [1, 0, 1],
        "m1": [[-1., 0., 1.], [1000., 1., 3.], [0., 0., 2.]],
        "m2": [[-1., 1., 2.], [1., 3., 0.], [0., 1., 2.]],
        "mat_expected": math.log(3.) + math.log(4.),
        "t1": [[[-1., 0., 1.], [1000., 1., 3.], [0., 0., 2.]], [[-1., 0., 1.], [1000., 1., 3.], [0., 0., 2.]]],
        "t2": [[[-1., 1., 0.], [1., 3., 0.], [0., 1., 2.]], [[-1., 1., 2.], [1., 3., 0.], [0., 1., 3.]]],
        "ten_expected": (math.log(1. + 3.) + math.log(4. + 6.)) - 2. * math.log(2.),
    }
    with open(os.path.join(HERE, "linear_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    write_jplace_fixture(ref_root)
    with open(os.path.join(HERE, "gamma_kat.json"), "w") as f:
        json.dump({"n_cat": 4, "alpha": 0.5,
                   "rates": [0.0333877533835995541, 0.251915917593438454, 0.820268481973647878,
                             2.89442784704931411]}, f, indent=1)


def jplace_tree_fixture(ref_root, rel):
    """The numbered reference tree of one of the reference's jplace test
    files: the tree without its edge numbers (parsed to post-order arrays)
    and the numbered string pplacer wrote, in version-3 braces."""
    with open(os.path.join(ref_root, rel)) as f:
        tree = json.load(f)["tree"]
    numbered = re.sub(r"\[(\d+)\]", r"{\1}", tree)  # version 1 wrote [n]
    plain = re.sub(r"\{\d+\}", "", numbered)
    parent, bl, label = parse_newick(plain)
    ids = [int(m) for m in re.findall(r"\{(\d+)\}", numbered)]
    assert sorted(ids) == list(range(len(parent)))
    return {"source": rel, "parent": parent, "bl": bl, "label": label, "numbered": numbered}


def write_jplace_fixture(ref_root):
    # tests/data/simple/test1.jplace (version 1) and tests/data/trim/trim_out.jplace (version 3)
    fx = [jplace_tree_fixture(ref_root, "tests/data/simple/test1.jplace"),
          jplace_tree_fixture(ref_root, "tests/data/trim/trim_out.jplace")]
    with open(os.path.join(HERE, "jplace_trees.json"), "w") as f:
        json.dump(fx, f, indent=1)
    # the placement rows of version-3 files written by pplacer's tools, as the
    # number tokens they hold (tests/data/misc/test_rarefy.jplace is left out:
    # its rows were written by hand, "1.0" / "0.0")
    rows = []
    for rel in ("tests/data/trim/trim_out.jplace", "tests/data/misc/test_indep_contrasts.jplace",
                "tests/data/misc/indep_scaled.jplace"):
        with open(os.path.join(ref_root, rel)) as f:
            txt = f.read()
        fields = json.loads(txt)["fields"]
        sec = txt[txt.index('"placements"'):txt.index('"metadata"')]
        toks = [[t.strip() for t in m.split(",")] for m in re.findall(r"\[([-0-9.eE+,\s]+)\]", sec)]
        rows.append({"source": rel, "fields": fields, "rows": toks})
    with open(os.path.join(HERE, "jplace_rows.json"), "w") as f:
        json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
