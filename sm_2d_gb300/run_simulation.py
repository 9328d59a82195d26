"""python -m sm_2d_gb300.run_simulation [sim.ini]: the reference's
run_simulation command (run_simulation.cpp:116-188) over the GB300 engine:
the INI file's spot, then dose_2d.txt and pdd.txt under its output_dir.  The
compiled command sm_2d_gb300/_lib/run_simulation does the same."""
import sys

from .runtime import Sm2dError, lib, run_simulation


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    ini = argv[0] if argv else "sim.ini"
    try:
        run_simulation(ini)
    except Sm2dError as e:
        print(f"Error: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    lib()
    sys.exit(main())
