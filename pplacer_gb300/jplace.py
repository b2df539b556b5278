"""jplace (version 3) output of placement results.

Restates the writer of pplacer_src/placerun_io.ml:58-90 (``to_json_file``)
with the pieces it calls:

* the placement fields of ``Placement.to_json`` (pplacer_src/placement.ml:
  168-175): edge_num, likelihood, like_weight_ratio, distal_length,
  pendant_length; the ``fields`` list is their sorted union
  (``StringSet.elements``, placerun_io.ml:81-83) and every ``p`` row lists the
  values in that order;
* ``Pquery_io.to_json`` (pplacer_src/pquery_io.ml:28-45): one object per
  query with ``p`` (its placements, best first) and ``nm`` ([name,
  multiplicity] pairs);
* the numbered reference tree of ``Newick_gtree.to_string
  ~with_node_numbers:true`` (pplacer_src/newick_gtree.ml:55-69,
  newick_bark.ml:18-30,74-79): ``label:%g{node}``, children in stored order,
  labels quoted as ``quote_label`` does;
* numbers as ``Json.to_formatter`` prints them (json_src/json.ml:40-43):
  integers with ``%d``, floats with ``%.12g``.

The top-level keys are written in the order pplacer's files show them
(tree, placements, metadata, version, fields); JSON readers do not depend on
it.
"""
import re

FIELDS = sorted(["edge_num", "likelihood", "like_weight_ratio", "distal_length", "pendant_length"])

_NEEDS_QUOTES = re.compile(r"[ \t\n(){}:;,\[\]'\\]")


def quote_label(s):
    """newick_bark.ml:18-30: quote a label holding Newick punctuation; ' and \\ are backslash-escaped."""
    if not _NEEDS_QUOTES.search(s):
        return s
    return "'" + re.sub(r"(['\\])", r"\\\1", s) + "'"


def _fmt_float(x):
    if x != x:
        return "nan"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    return "%.12g" % x


def numbered_newick(parent, bl, labels=None):
    """Newick string of a tree in pplacer's post-order numbering, every node
    followed by ``{id}`` after its branch length; children in increasing id
    order (the order of the original Newick string)."""
    n = len(parent)
    children = [[] for _ in range(n)]
    root = -1
    for i, p in enumerate(parent):
        if p < 0:
            root = i
        else:
            children[p].append(i)
    if root < 0:
        raise ValueError("tree without a root")

    def bark(i):
        lab = quote_label(labels[i]) if labels is not None and labels[i] else ""
        return "%s:%s{%d}" % (lab, "%g" % bl[i], i)

    # iterative post-order to stay clear of the recursion limit on deep trees
    out = {}
    stack = [(root, False)]
    while stack:
        i, done = stack.pop()
        if not children[i]:
            out[i] = bark(i)
        elif done:
            out[i] = "(" + ",".join(out.pop(c) for c in sorted(children[i])) + ")" + bark(i)
        else:
            stack.append((i, True))
            stack.extend((c, False) for c in children[i])
    return out[root] + ";"


def _dump(v, out):
    if isinstance(v, bool):
        out.append("true" if v else "false")
    elif isinstance(v, int):
        out.append("%d" % v)
    elif isinstance(v, float):
        out.append(_fmt_float(v))
    elif isinstance(v, str):
        out.append('"' + v.replace("\\", "\\\\").replace('"', '\\"').replace("/", "\\/")
                   .replace("\n", "\\n").replace("\r", "\\r").replace("\t", "\\t") + '"')
    elif isinstance(v, dict):
        out.append("{")
        for k, (key, val) in enumerate(v.items()):
            if k:
                out.append(", ")
            _dump(key, out)
            out.append(": ")
            _dump(val, out)
        out.append("}")
    elif isinstance(v, (list, tuple)):
        out.append("[")
        for k, val in enumerate(v):
            if k:
                out.append(", ")
            _dump(val, out)
        out.append("]")
    elif v is None:
        out.append("null")
    else:
        raise TypeError(type(v))


def to_jplace(results, names, parent, bl, labels=None, invocation="pplacer_gb300"):
    """The jplace text of placement results.

    results: per query, a list of (edge, like, lwr, distal, pendant) tuples
    best first (Engine.place / Engine.fetch), or (..., post_prob,
    marginal_like) with posterior probabilities, which adds those two fields
    (placement.ml:176-180); queries with no placement are left out, as
    pplacer leaves out failed queries.  names: per query a name, or a list
    of names (``model.dedup``), each written with multiplicity 1
    (placerun.ml:95-112)."""
    rows = []
    with_pp = any(len(pl) > 5 for places in results for pl in places)
    fields = sorted(FIELDS + (["marginal_like", "post_prob"] if with_pp else []))
    for name, places in zip(names, results):
        if not places:
            continue
        p = []
        for pl in places:
            edge, like, lwr, dist, pend = pl[:5]
            val = {"edge_num": int(edge), "likelihood": float(like), "like_weight_ratio": float(lwr),
                   "distal_length": float(dist), "pendant_length": float(pend)}
            if with_pp:
                val["post_prob"], val["marginal_like"] = float(pl[5]), float(pl[6])
            p.append([val[f] for f in fields])
        namel = [name] if isinstance(name, str) else list(name)
        rows.append({"p": p, "nm": [[n, 1] for n in namel]})
    doc = {"tree": numbered_newick(parent, bl, labels), "placements": rows,
           "metadata": {"invocation": invocation}, "version": 3, "fields": fields}
    out = []
    _dump(doc, out)
    return "".join(out) + "\n"


def write_jplace(path, results, names, parent, bl, labels=None, invocation="pplacer_gb300"):
    with open(path, "w") as f:
        f.write(to_jplace(results, names, parent, bl, labels, invocation))
