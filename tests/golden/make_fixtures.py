"""Regenerate the golden fixtures from the reference checkout.

Run in a container where the reference project is mounted (it does not exist
on the GPU machines, so the outputs are committed):

    python tests/golden/make_fixtures.py /path/to/reference

(or with the checkout's path in the environment variable RSD_REFERENCE).

Writes
  tests/golden/tablefar_equal.txt  the equal-sphere rows (lambda = 1) of the
      reference's own output table src/lubrication tabel/FarfieldForce/
      tablefar.txt: free-space two-sphere resistance functions obtained by
      inverting the grand RPY mobility with MATREV.  They pin the oracle's
      pair tensors, Y2 projection and SPD inversion.
  tests/golden/lubdat/{r2babc,r2bgh,r2bm}.dat  the lubrication tables the
      reference reads at run time (examples/lubdat), byte for byte; they
      are inputs of lubmxcalc, kept in the reference's own file format so
      the C-ABI loader reads the same files a Fortran run reads.
  tests/golden/io/{control_file.dat,initial_config.dat}  the reference's
      example driver inputs (examples/), byte for byte, and
  tests/golden/io/output_head.VTF  the first 40 records of its example
      trajectory output (examples/gmmres_output.VTF), for the readers and
      writers of the driver's file formats.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    src = os.path.join(ref, "src", "lubrication tabel", "FarfieldForce", "tablefar.txt")
    rows = []
    with open(src) as fp:
        header = fp.readline()
        for line in fp:
            v = line.split()
            if len(v) == 24 and float(v[0]) == 1.0:
                rows.append(line.rstrip("\n"))
    with open(os.path.join(HERE, "tablefar_equal.txt"), "w") as fp:
        fp.write("# equal-sphere rows of the reference's src/lubrication tabel/FarfieldForce/tablefar.txt\n")
        fp.write("# columns: " + " ".join(header.split()) + "\n")
        fp.write("\n".join(rows) + "\n")
    os.makedirs(os.path.join(HERE, "lubdat"), exist_ok=True)
    for name in ("r2babc.dat", "r2bgh.dat", "r2bm.dat"):
        shutil.copyfile(os.path.join(ref, "examples", "lubdat", name), os.path.join(HERE, "lubdat", name))
    os.makedirs(os.path.join(HERE, "io"), exist_ok=True)
    for name in ("control_file.dat", "initial_config.dat"):
        shutil.copyfile(os.path.join(ref, "examples", name), os.path.join(HERE, "io", name))
    with open(os.path.join(ref, "examples", "gmmres_output.VTF")) as fp:
        head = [fp.readline() for _ in range(40)]
    with open(os.path.join(HERE, "io", "output_head.VTF"), "w") as fp:
        fp.write("".join(head))
    print("wrote %d tablefar rows, 3 lubrication tables and the driver file fixtures" % len(rows))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RSD_REFERENCE")
    if not ref:
        sys.exit("usage: make_fixtures.py <reference checkout> (or set RSD_REFERENCE)")
    main(ref)
