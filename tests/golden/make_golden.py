"""Copy the golden data of Typhon's non-regression suite used by the tests.

Run once in a container where the reference checkout is mounted (default path
below, or pass it as the first argument).  It copies, unchanged:

* the XBIN/TYPHON meshes of NRG/COMMON that the cases use (``*.tym``);
* the monitor files written by Typhon for those cases (``*.tmon``), renamed
  ``<case>__<file>``.

The copies are committed so that the tests never read the reference at run time.
"""
import pathlib
import shutil
import sys

REF = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
HERE = pathlib.Path(__file__).resolve().parent

MESHES = ["quad20x20.tym", "quad20x10.tym", "quad10x10.tym", "tri5x10.tym", "mxlay2x20quad-h50.tym"]
CASES = {
    "RK2": "NRG/TIME/RUNGEKUTTA/RK2/RHOERR.tmon",
    "RK2-SSP": "NRG/TIME/RUNGEKUTTA/RK2-SSP/RHOERR.tmon",
    "RK3-SSP": "NRG/TIME/RUNGEKUTTA/RK3-SSP/RHOERR.tmon",
    "RK4": "NRG/TIME/RUNGEKUTTA/RK4/RHOERR.tmon",
    "RK25BB": "NRG/TIME/RUNGEKUTTA/RK25BB/RHOERR.tmon",
    "RK26BB": "NRG/TIME/RUNGEKUTTA/RK26BB/RHOERR.tmon",
    "RK12BS": "NRG/TIME/RUNGEKUTTA/RK12BS/RHOERR.tmon",
    "RK13BS": "NRG/TIME/RUNGEKUTTA/RK13BS/RHOERR.tmon",
    "PER2D-TRANS": "NRG/MESH/CON/PER2D-TRANS/RHODEV.tmon",
    "TYM-QUAD": "NRG/MESH/ELEM/TYM-QUAD/PAVG.tmon",
    "VISCOUS-CELLAVG-DELTA": "NRG/NS/NUM/FLUX/VISCOUS/CELLAVG/DELTA.tmon",
    "VISCOUS-CELLAVG-VXERR": "NRG/NS/NUM/FLUX/VISCOUS/CELLAVG/VXERR.tmon",
    "VISCOUS-CELLFULL-DELTA": "NRG/NS/NUM/FLUX/VISCOUS/CELLFULL/DELTA.tmon",
    "VISCOUS-CELLFULL-VXERR": "NRG/NS/NUM/FLUX/VISCOUS/CELLFULL/VXERR.tmon",
}

def main():
    for m in MESHES:
        shutil.copyfile(REF / "NRG/COMMON" / m, HERE / m)
    for name, rel in CASES.items():
        src = REF / rel
        shutil.copyfile(src, HERE / f"{name}__{src.name}")
    print("copied", len(MESHES), "meshes and", len(CASES), "monitor files into", HERE)

if __name__ == "__main__":
    main()
