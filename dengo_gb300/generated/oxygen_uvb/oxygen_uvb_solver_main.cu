/* THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.
 *
 * Stand-alone driver of network "oxygen_uvb" (the reference's
 * rates_and_rate_tables_main.C.template): oxygen_uvb_initial_conditions.dgt
 * -> oxygen_uvb_solution.dgt, in the current directory or in argv[1].
 *
 *   nvcc -o oxygen_uvb_main oxygen_uvb_solver_main.cu -I <package>/include -I . \
 *        -L . -loxygen_uvb_solver -Xlinker -rpath -Xlinker .
 */
#include <stdio.h>

#include "oxygen_uvb_solver.h"

int main(int argc, char **argv)
{
    const int rc = oxygen_uvb_main(argc, argv);
    if (rc != 0) fprintf(stderr, "oxygen_uvb_main: %s\n", oxygen_uvb_last_error());
    return rc;
}
