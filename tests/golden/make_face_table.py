"""Extract the face re-orientation table golden fixture from the reference.

TSEMLib reads `include/quad_info/Info_Interpolate_More` (record layout in
src/BuildSpace.cpp:1704-1771): a header M_tmp, then for each of the 6 vertex
permutations of a face and each face DOF (ordered by total degree) three edge
records and one face record, each `count (index value)*`.  Face DOFs of total
degree <= M only reference DOFs of degree <= M, so the first nf(M) records of
every permutation form the complete table for order M.

This script writes that prefix for M = 10 (the largest order any configuration
uses is 8; the oracle reads this one) as `face_table_M10.txt`, and for M = 16 (the
largest order the library accepts) as `face_table_M16.txt`, in the same layout.  It
is the only place the reference tree is read; run it in a checkout that has the
reference available:

    python tests/golden/make_face_table.py /path/to/TSEMLib
"""
import os
import sys

M_OUTS = (10, 16)


def nface(m):
    return (m - 2) * (m - 3) // 2 + m - 2


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_face_table.py <path of the TSEMLib checkout>")
    ref = sys.argv[1]
    src = os.path.join(ref, "include", "quad_info", "Info_Interpolate_More")
    tok = open(src).read().split()
    pos = 0
    m_in = int(tok[pos]); pos += 1
    nf_in = nface(m_in)
    edge_recs, face_recs = [], []          # per permutation
    for _var in range(6):
        edges, faces = [], []
        for d in range(nf_in):
            recs = []
            for _e in range(3):
                c = int(tok[pos]); pos += 1
                ent = [(int(tok[pos + 2 * i]), tok[pos + 2 * i + 1]) for i in range(c)]
                pos += 2 * c
                recs.append(ent)
            edges.append(recs)
        for d in range(nf_in):
            c = int(tok[pos]); pos += 1
            ent = [(int(tok[pos + 2 * i]), tok[pos + 2 * i + 1]) for i in range(c)]
            pos += 2 * c
            faces.append(ent)
        edge_recs.append(edges)
        face_recs.append(faces)
    assert pos == len(tok)
    for m_out in M_OUTS:
        nf_out = nface(m_out)
        out = [str(m_out)]
        for var in range(6):
            for d in range(nf_out):
                for ent in edge_recs[var][d]:
                    assert all(i <= m_out - 2 for i, _ in ent), "edge index beyond order"
                    out.append(" ".join([str(len(ent))] + [f"{i} {v}" for i, v in ent]))
            for d in range(nf_out):
                ent = face_recs[var][d]
                assert all(i < nf_out for i, _ in ent), "face index beyond order"
                out.append(" ".join([str(len(ent))] + [f"{i} {v}" for i, v in ent]))
        dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), f"face_table_M{m_out}.txt")
        with open(dst, "w") as f:
            f.write("\n".join(out) + "\n")
        print("wrote", dst)


if __name__ == "__main__":
    main()
