/* THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.
 *
 * Stand-alone driver of network "primordial_compton" (the reference's
 * rates_and_rate_tables_main.C.template): primordial_compton_initial_conditions.dgt
 * -> primordial_compton_solution.dgt, in the current directory or in argv[1].
 *
 *   nvcc -o primordial_compton_main primordial_compton_solver_main.cu -I <package>/include -I . \
 *        -L . -lprimordial_compton_solver -Xlinker -rpath -Xlinker .
 */
#include <stdio.h>

#include "primordial_compton_solver.h"

int main(int argc, char **argv)
{
    const int rc = primordial_compton_main(argc, argv);
    if (rc != 0) fprintf(stderr, "primordial_compton_main: %s\n", primordial_compton_last_error());
    return rc;
}
