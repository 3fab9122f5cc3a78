"""Graph file conversion, as the reference's convert example
(examples/convert/convert.cpp:1-33): read a graph in one of the reference's
formats and write it as an edge list ("source target" per CSR entry), or, with
--csr, as the binary CSR cache that gu_hgraph_parse(..., "csrbin") reads back.

    python graph-utils_gb300/convert.py -i graph.metis -f dimacs -o graph.txt
    python graph-utils_gb300/convert.py -i graph.metis -f dimacs -o graph.csr --csr
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import gu  # noqa: E402


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("-i", "--infile", required=True)
    p.add_argument("-f", "--format", required=True, help="dimacs, edgelist, edgelist_h, market or csrbin")
    p.add_argument("-o", "--outfile")
    p.add_argument("--csr", action="store_true", help="write the binary CSR cache instead of an edge list")
    p.add_argument("--header", action="store_true", help="edge list: first line 'n m'")
    a = p.parse_args(argv)
    g = gu.HostGraph.parse(a.infile, a.format)
    print("Graph parsed.")
    print(f"Number of vertices: {g.n}")
    print(f"Number of (directed) edges: {g.m}")
    print(f"Vertices of degree zero: {g.count_degree_zero()}")
    if not a.outfile:
        print("Error: Cannot convert graph since no output file was given. Use -o to name one.", file=sys.stderr)
        return 1
    if a.csr:
        g.write_csr(a.outfile)
    else:
        g.write_edgelist(a.outfile, header=a.header)
    print("Conversion successful")
    return 0


if __name__ == "__main__":
    sys.exit(main())
