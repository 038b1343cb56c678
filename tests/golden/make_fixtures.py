"""Generate the golden fixtures of the tests from the reference tree.

Run here (where the reference is mounted); the outputs are committed so the
tests never read the reference at run time:

  materials.json  Filmetrics n,k tables the reference's unit tests load
                  (tutorials/{Al,Si,Si3N4,SiO2,TiO2}.txt)
  glasses.agf     the N-BK7 and LITHOSIL-Q records of
                  misc/schottzemax-20180601.agf (NM/CD/IT lines)

  python tests/golden/make_fixtures.py /root/reference
"""
import json
import os
import sys


def filmetrics(path):
    wl, n, k = [], [], []
    with open(path, encoding="utf-8-sig") as f:
        head = f.readline().strip()
        assert head == "Wavelength(nm)\tn\tk", head
        for line in f:
            p = line.split()
            if len(p) >= 3:
                wl.append(float(p[0]))
                n.append(float(p[1]))
                k.append(float(p[2]))
    return {"wavelength_nm": wl, "n": n, "k": k}


def agf_records(path, names):
    out, keep = [], False
    with open(path, encoding="latin-1") as f:
        for line in f:
            if line.startswith("NM "):
                keep = line.split()[1] in names
            if keep and line[:3] in ("NM ", "CD ", "IT "):
                out.append(line.rstrip() + "\n")
    return out


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    mats = {m: filmetrics(os.path.join(ref, "tutorials", f"{m}.txt")) for m in ("Al", "Si", "Si3N4", "SiO2", "TiO2")}
    with open(os.path.join(here, "materials.json"), "w") as f:
        json.dump(mats, f)
    recs = agf_records(os.path.join(ref, "misc", "schottzemax-20180601.agf"), {"N-BK7", "LITHOSIL-Q"})
    with open(os.path.join(here, "glasses.agf"), "w") as f:
        f.writelines(recs)
    print("wrote", len(mats), "materials and", len(recs), "catalog lines")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
