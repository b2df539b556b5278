"""jplace writer (placerun_io.ml:58-90): numbered tree strings against the
reference's own jplace test files, field order, number formatting."""
import json
import os

from pplacer_gb300 import jplace

GOLD = os.path.join(os.path.dirname(__file__), "golden", "jplace_trees.json")


def test_numbered_tree_matches_reference_files():
    for fx in json.load(open(GOLD)):
        got = jplace.numbered_newick(fx["parent"], fx["bl"], fx["label"])
        assert got == fx["numbered"], fx["source"]


def test_quote_label():
    assert jplace.quote_label("taxon_1") == "taxon_1"
    assert jplace.quote_label("a b") == "'a b'"
    assert jplace.quote_label("x(1)") == "'x(1)'"
    assert jplace.quote_label("it's") == "'it\\'s'"
    assert jplace.quote_label("a\\b") == "'a\\\\b'"


def test_document_layout():
    parent, bl = [2, 2, -1], [0.1, 0.25, 0.0]
    results = [[(0, -1309.83, 0.710949502625, 0.5, 0.9), (1, -1310.1, 0.289050497375, 1.0, 2.4)], [],
               [(1, -20.0, 1.0, 0.125, 1e-08)]]
    text = jplace.to_jplace(results, ["q1", "q2", "q3"], parent, bl, ["A", "B", ""], invocation="test run")
    doc = json.loads(text)
    assert list(doc) == ["tree", "placements", "metadata", "version", "fields"]
    assert doc["version"] == 3
    assert doc["fields"] == ["distal_length", "edge_num", "like_weight_ratio", "likelihood", "pendant_length"]
    assert doc["tree"] == "(A:0.1{0},B:0.25{1}):0{2};"
    assert doc["metadata"] == {"invocation": "test run"}
    # the query without placements is left out; rows follow the field order
    assert [r["nm"] for r in doc["placements"]] == [[["q1", 1]], [["q3", 1]]]
    assert doc["placements"][0]["p"][0] == [0.5, 0, 0.710949502625, -1309.83, 0.9]
    assert "-1309.83," in text and "1e-08" in text  # %.12g numbers, %d edge numbers
    assert "0.710949502625" in text


def test_dedup_and_redup():
    from pplacer_gb300.model import dedup
    names = ["a", "b", "c", "d", "e"]
    seqs = ["ACGT", "AC-T", "ACGT", "ACGT", "AC-T"]
    uniq, namel = dedup(names, seqs)
    assert uniq == ["ACGT", "AC-T"]
    assert namel == [["a", "c", "d"], ["b", "e"]]
    results = [[(0, -10.0, 1.0, 0.05, 0.1)], [(1, -12.0, 1.0, 0.025, 0.2)]]
    doc = json.loads(jplace.to_jplace(results, namel, [2, 2, -1], [0.1, 0.05, 0.0], ["A", "B", ""]))
    assert [r["nm"] for r in doc["placements"]] == [[["a", 1], ["c", 1], ["d", 1]], [["b", 1], ["e", 1]]]
    try:
        dedup(["a"], ["A", "C"])
    except ValueError:
        pass
    else:
        raise AssertionError("length mismatch accepted")


def test_posterior_fields():
    """Placements with posterior probabilities add marginal_like and
    post_prob to the sorted field list (placement.ml:176-180)."""
    parent, bl = [2, 2, -1], [0.1, 0.25, 0.0]
    results = [[(0, -10.0, 0.75, 0.05, 0.1, 0.8, -12.5), (1, -11.1, 0.25, 0.1, 0.2, 0.2, -13.9)]]
    doc = json.loads(jplace.to_jplace(results, ["q"], parent, bl))
    assert doc["fields"] == ["distal_length", "edge_num", "like_weight_ratio", "likelihood", "marginal_like",
                             "pendant_length", "post_prob"]
    assert doc["placements"][0]["p"][0] == [0.05, 0, 0.75, -10.0, -12.5, 0.1, 0.8]


def test_numbers_as_pplacer_writes_them():
    """The placement rows of version-3 files written by pplacer's tools: each
    number the writer emits for the parsed values is the token in the file
    (%d edge numbers, %.12g floats, json.ml:40-43)."""
    import re
    rows = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "jplace_rows.json")))
    n = 0
    for fx in rows:
        fields = fx["fields"]
        results = []
        for toks in fx["rows"]:
            vals = dict(zip(fields, toks))
            results.append([(int(vals["edge_num"]), float(vals["likelihood"]), float(vals["like_weight_ratio"]),
                             float(vals["distal_length"]), float(vals["pendant_length"]))])
        text = jplace.to_jplace(results, ["q%d" % i for i in range(len(results))], [1, -1], [0.5, 0.0])
        emitted = [[t.strip() for t in m.split(",")]
                   for m in re.findall(r"\[([-0-9.eE+,\s]+)\]", text[text.index('"placements"'):text.index('"metadata"')])]
        assert len(emitted) == len(fx["rows"]), fx["source"]
        for toks, out in zip(fx["rows"], emitted):
            want = dict(zip(fields, toks))
            got = dict(zip(jplace.FIELDS, out))
            assert got == want, (fx["source"], got, want)
            n += 1
    assert n >= 25
