/* run_simulation: the reference's command-line entry (run_simulation.cpp:116-188)
 * over libsm2d.so, so that batch drivers that call `run_simulation <ini>` run
 * the GB300 engine unchanged.  Exit status 0 on success, 1 with the error on
 * stderr otherwise. */
#include <stdio.h>

#include "sm2d.h"

int main(int argc, char** argv) {
    const char* ini = argc > 1 ? argv[1] : "sim.ini";
    printf("SM_2D (GB300): configuration %s\n", ini);
    if (sm2d_run_simulation(ini) != 0) {
        fprintf(stderr, "Error: %s\n", sm2d_last_error());
        return 1;
    }
    return 0;
}
