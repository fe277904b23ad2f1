"""Copy the golden data of Typhon's non-regression suite used by the tests.

Run once where a checkout of the reference is available, with its path as the only
argument (``python tests/golden/make_golden.py <typhon checkout>``).  It copies, unchanged:

* the XBIN/TYPHON meshes of NRG/COMMON that the cases use (``*.tym``) and the CGNS
  (ADF) meshes of the implicit and heat-conduction cases (``*.cgns``);
* the monitor files written by Typhon for those cases (``*.tmon``, residual histories
  ``monres.*``, boundary histories ``histo*``) and one VTK output file, renamed
  ``<case>__<file>``.

The copies are committed so that the tests never read the reference at run time.
"""
import pathlib
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <path of the Typhon checkout>")
REF = pathlib.Path(sys.argv[1])
HERE = pathlib.Path(__file__).resolve().parent

MESHES = ["quad20x20.tym", "quad20x10.tym", "quad10x10.tym", "tri5x10.tym", "mxlay2x20quad-h50.tym",
          "tube.cgns", "square-quad10.cgns", "rect4x1.cgns", "expansion-10.cgns", "perrot2d.cgns"]
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
    "PER2D-ROT": ["NRG/MESH/CON/PER2D-ROT/histovarNS_RMIN", "NRG/MESH/CON/PER2D-ROT/histovarNS_RMAX"],
    "TYM-QUAD": "NRG/MESH/ELEM/TYM-QUAD/PAVG.tmon",
    "VISCOUS-CELLAVG-DELTA": "NRG/NS/NUM/FLUX/VISCOUS/CELLAVG/DELTA.tmon",
    "VISCOUS-CELLAVG-VXERR": "NRG/NS/NUM/FLUX/VISCOUS/CELLAVG/VXERR.tmon",
    "VISCOUS-CELLFULL-DELTA": "NRG/NS/NUM/FLUX/VISCOUS/CELLFULL/DELTA.tmon",
    "VISCOUS-CELLFULL-VXERR": "NRG/NS/NUM/FLUX/VISCOUS/CELLFULL/VXERR.tmon",
    "KDIF-ISOTH-CGS": ["NRG/KDIF/ISOTH-CGS/monres.001", "NRG/KDIF/ISOTH-CGS/Average_T.tmon"],
    "KDIF-ISOTH-GMRES": ["NRG/KDIF/ISOTH-GMRES/monres.001", "NRG/KDIF/ISOTH-GMRES/Average_T.tmon"],
    "KDIF-ISOTH-BICG": ["NRG/KDIF/ISOTH-BICG/monres.001", "NRG/KDIF/ISOTH-BICG/Average_T.tmon"],
    "IMPLICIT-GMRES": ["NRG/TIME/IMPLICIT/GMRES/histofluxNS_RIGHT", "NRG/TIME/IMPLICIT/GMRES/histovarNS_RIGHT"],
    "IMPLICIT-BICGSTAB-RUSANOV": ["NRG/TIME/IMPLICIT/BICGSTAB-RUSANOV/histovarNS_DOWN"],
    "HLLC-MUSCL": "NRG/NS/NUM/HRES/MUSCL/HLLC-MUSCL/monres.001",
    "HLLC-MUSCLUNS": "NRG/NS/NUM/FLUX/HLLC-MUSCLUNS/monres.001",
    "HLLC-MPI": "NRG/NS/HLLC-MPI/monres.001",
    "HLLE-EXPLICIT": ["NRG/NS/NUM/FLUX/HLLE/histofluxNS_RIGHT", "NRG/NS/NUM/FLUX/HLLE/histovarNS_RIGHT"],
    "AUSM-MUSCLFAST": ["NRG/NS/NUM/HRES/MUSCL/AUSM-MUSCLFAST/monres.001",
                       "NRG/NS/NUM/HRES/MUSCL/AUSM-MUSCLFAST/typhonNS.vtk"],
    "AUSM-MUSCLUNS": ["NRG/NS/NUM/HRES/MUSCL/AUSM-MUSCLUNS/MAXV.tmon",
                      "NRG/NS/NUM/HRES/MUSCL/AUSM-MUSCLUNS/MINP.tmon",
                      "NRG/NS/NUM/HRES/MUSCL/AUSM-MUSCLUNS/VCOMP.tmon"],
}

def main():
    for m in MESHES:
        shutil.copyfile(REF / "NRG/COMMON" / m, HERE / m)
    for name, rels in CASES.items():
        for rel in [rels] if isinstance(rels, str) else rels:
            src = REF / rel
            shutil.copyfile(src, HERE / f"{name}__{src.name}")
    print("copied", len(MESHES), "meshes and", len(CASES), "monitor files into", HERE)

if __name__ == "__main__":
    main()
