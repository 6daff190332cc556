"""VQL front end: the parser (no GPU) on the reference's own example queries
and on each grammar form (src/objects/vql/grammar/vql.g4,
src/objects/vql/vql-interface.cpp, query_builder.cpp:294-304)."""
import ctypes as C

import pytest

from vertexsurge_gb300 import build


@pytest.fixture(scope="module")
def ops():
    build.build_all()
    lib = C.CDLL(str(build.OPS_LIB))
    lib.vsops_vql_describe.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
    lib.vsops_vql_describe.restype = C.c_int
    return lib


def describe(ops, q):
    buf = C.create_string_buffer(4096)
    rc = ops.vsops_vql_describe(q.encode(), buf, len(buf))
    return rc, buf.value.decode()


def test_reference_example_queries(ops):
    rc, d = describe(ops, "vmatch (a{tag:1-1})->(b), (b{tag:3-3})<-[2..4]-(c{tag:2-2})-[]s-(a) "
                          "return a.id,b.community,c;")
    assert rc == 0, d
    assert d == ("V a:TAG:1-1 b:TAG:3-3 c:TAG:2-2 | E a>b:F:1-1:any b>c:B:2-4:any c>a:U:1-1:shortest "
                 "| R a.id b.community c")
    rc, d = describe(ops, "vmatch (a{tag:1-1})->(b), (b{tag:1-100})<-[2..4]-(c{id:1})-[]s-(a) "
                          "return a.id,b.community,c;")
    assert rc == 0 and "c:ID:1" in d and "b:TAG:1-100" in d


@pytest.mark.parametrize("q,edges", [
    ("vmatch (a)->(b) return count of a, b;", "a>b:F:1-1:any"),
    ("vmatch (a)<-(b) return a;", "a>b:B:1-1:any"),
    ("vmatch (a)-(b) return a;", "a>b:U:1-1:any"),
    ("vmatch (a)-[3]->(b) return a;", "a>b:F:3-3:any"),
    ("vmatch (a)-[2..5]s->(b) return a;", "a>b:F:2-5:shortest"),
    ("vmatch (a)<-[1..2]s-(b) return a;", "a>b:B:1-2:shortest"),
    ("vmatch (a)-[0..3]-(b) return a;", "a>b:U:0-3:any"),
    ("vmatch (x_1)-[]-(y2)-[2]-(x_1) return x_1;", "x_1>y2:U:1-1:any y2>x_1:U:2-2:any"),
])
def test_edge_forms(ops, q, edges):
    rc, d = describe(ops, q)
    assert rc == 0, d
    assert d.split(" | ")[1] == "E " + edges
    assert d.endswith("| count") == ("count of" in q)


@pytest.mark.parametrize("q", [
    "vmatch (a)->(b) return a",                 # no ';'
    "vmatch (a)-[..3]->(b) return a;",          # variable length without a start
    "vmatch (a)-[4..2]->(b) return a;",         # start above end
    "vmatch (a{tag:1})->(b) return a;",         # tag needs a range
    "vmatch (a{tag:1-1})->(a{tag:2-2}) return a;",  # two filters on one vertex
    "match (a)->(b) return a;",
    "vmatch (a)->(b) return a; extra",
])
def test_syntax_errors(ops, q):
    rc, d = describe(ops, q)
    assert rc != 0 and d
