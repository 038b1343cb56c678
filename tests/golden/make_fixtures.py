"""Generate the golden fixtures of the tests from the reference tree.

Run here (where the reference is mounted); the outputs are committed so the
tests never read the reference at run time:

  materials.json  Filmetrics n,k tables the reference's unit tests load
                  (tutorials/{Al,Si,Si3N4,SiO2,TiO2}.txt)
  glasses.agf     the N-BK7 and LITHOSIL-Q records of
                  misc/schottzemax-20180601.agf (NM/CD/IT lines)
  muon_ring4.corsika.gz
                  the CORSIKA IACT event of tutorials/CORSIKA.C (data file,
                  copied as is)
  corsika_muon_ring4.npz
                  what the reference's own eventio reader (src/bernlohr,
                  compiled by oracle/build_ref.sh into oracle/_ref) reads
                  from it: run header, input-card line count, telescope
                  positions, event header, array offsets and every bunch

  python tests/golden/make_fixtures.py REFERENCE_ROOT

REFERENCE_ROOT defaults to $ROBAST_REFERENCE, else to a checkout named
"reference" beside this repository.
"""
import json
import os
import shutil
import subprocess
import sys

import numpy as np


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


def corsika_dump(ref, here):
    """Parse the text dump of oracle/_ref/corsika_dump (one event)."""
    root = os.path.dirname(os.path.dirname(here))
    subprocess.run([os.path.join(root, "oracle", "build_ref.sh"), ref], check=True, stdout=subprocess.DEVNULL)
    src = os.path.join(ref, "tutorials", "muon_ring4.corsika.gz")
    shutil.copyfile(src, os.path.join(here, "muon_ring4.corsika.gz"))
    txt = subprocess.run([os.path.join(root, "oracle", "_ref", "corsika_dump"), src], check=True,
                         capture_output=True, text=True).stdout.splitlines()
    out = {"tel": [], "bunch": [], "bunch_tel": [], "bunch_array": [], "offsets": []}
    cur = None
    for line in txt:
        p = line.split()
        if p[0] in ("RUNH", "EVTH"):
            # word 0 is the record tag (int32 bits), printed as the float
            # those bits make; compare words 1.. only
            out[p[0].lower()] = np.array([float(v) for v in p[2:]], dtype=np.float32)
        elif p[0] == "INPUT":
            out["input_lines"] = int(p[1])
        elif p[0] == "TEL":
            out["tel"].append([float(v) for v in p[1:5]])
        elif p[0] == "TELOFF":
            out["time_offset"] = float(p[2])
        elif p[0] == "OFF":
            out["offsets"].append([float(v) for v in p[1:3]])
        elif p[0] == "PHOTONS":
            cur = (int(p[1]), int(p[2]))
        elif p[0] == "B":
            out["bunch"].append([float(v) for v in p[1:9]])
            out["bunch_array"].append(cur[0])
            out["bunch_tel"].append(cur[1])
    np.savez_compressed(os.path.join(here, "corsika_muon_ring4.npz"), runh=out["runh"], evth=out["evth"],
                        input_lines=out["input_lines"], tel=np.array(out["tel"]), time_offset=out["time_offset"],
                        offsets=np.array(out["offsets"]),
                        bunch=np.array(out["bunch"], dtype=np.float32),
                        bunch_tel=np.array(out["bunch_tel"], dtype=np.int32),
                        bunch_array=np.array(out["bunch_array"], dtype=np.int32))
    return len(out["bunch"])


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    mats = {m: filmetrics(os.path.join(ref, "tutorials", f"{m}.txt")) for m in ("Al", "Si", "Si3N4", "SiO2", "TiO2")}
    with open(os.path.join(here, "materials.json"), "w") as f:
        json.dump(mats, f)
    recs = agf_records(os.path.join(ref, "misc", "schottzemax-20180601.agf"), {"N-BK7", "LITHOSIL-Q"})
    with open(os.path.join(here, "glasses.agf"), "w") as f:
        f.writelines(recs)
    nb = corsika_dump(ref, here)
    print("wrote", len(mats), "materials,", len(recs), "catalog lines and", nb, "CORSIKA bunches")


if __name__ == "__main__":
    default = os.environ.get("ROBAST_REFERENCE") or os.path.join(
        os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference")
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.normpath(default))
