"""The graph-simulation input readers follow the reference's parsing
(graphsim.cpp:14-40, graphsim_query.h:17-52), quirks included.  CPU only."""
import la3_gb300 as L


def test_data_labels(tmp_path):
    p = tmp_path / "d.labels"
    p.write_text('[\n{"d":"edu"},\n{"name":"x y"},\n{"k":""},\n{"a":"b":"c"},\n]\n')
    # an empty label: strtok skips the leading quote, so the label is '},'
    assert L.read_graphsim_labels(p, 4) == ["edu", "x y", "},", "b"]
    p.write_text('[\nnull,\n{"d":"P"},\n]\n')
    assert L.read_graphsim_labels(p, 2) == ["", "P"]
    # more vertices than lines: the missing ones stay unlabelled
    assert L.read_graphsim_labels(p, 4) == ["", "P", "", ""]


def test_query_labels_and_edges(tmp_path):
    lab, mtx = tmp_path / "q.labels", tmp_path / "q.mtx"
    mtx.write_text("0 1\n1 2\n2 0")
    lab.write_text("A\nB\nC")          # no trailing newline: three labels
    assert L.read_graphsim_query(lab, mtx) == (["A", "B", "C"], [(0, 1), (1, 2), (2, 0)])
    lab.write_text("A B\nC\n")         # trailing whitespace: one more, empty, label
    assert L.read_graphsim_query(lab, mtx)[0] == ["A", "B", "C", ""]
    lab.write_text("")                  # nothing: one empty label
    assert L.read_graphsim_query(lab, mtx)[0] == [""]
    mtx.write_text("0 1\n\n1 0\n")
    assert L.read_graphsim_query(lab, mtx)[1] == [(0, 1), (1, 0)]


def test_label_ids():
    v, q = L.graphsim_label_ids(["A", "", "B", "A"], ["B", "", "Z"], 5)
    assert v.tolist()[:4] == [v[0], 0, v[2], v[0]] and v[4] == 0
    assert q[0] == v[2] and q[1] == 0 and q[2] not in set(v.tolist())
