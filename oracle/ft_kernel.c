/*
 * ft_kernel.c -- one OpenCL program rendered by the reference
 * FiberTissueSimulation (myokit/_sim/openclsim.cl with fiber_tissue set for
 * the fiber), compiled as C, with its NDRange launches written as loops over
 * work items for the oracle's fiber-tissue host loop (oracle/ft_backend.py).
 *
 * TEST INFRASTRUCTURE (the oracle): used only by tests/, never by the
 * product.
 *
 * Compiled once per kernel source:
 *   gcc -O2 -std=gnu99 -fPIC -shared -ffp-contract=off
 *       -DORC_KERNEL='"<kernel>.cl"' [-DFTK_JUNCTION] ft_kernel.c -lm
 * FTK_JUNCTION: the program also holds diff_step_fiber_tissue (the fiber's).
 *
 * The time, step and pacing arguments arrive as doubles already rounded to
 * the kernel precision by the caller, as fiber_tissue.c rounds arg_time,
 * arg_dt and arg_pace (fiber_tissue.c:1030, 1126-1133).
 */
#include <math.h>
#include <stdlib.h>

#include "oracle_shim.h"
#include ORC_KERNEL

__thread unsigned long orc_gid[2];

int ftk_real_bytes(void) { return (int)sizeof(Real); }

/* diff_step over an nx x ny grid (openclsim.cl:384-435) */
void ftk_diff(long nx, long ny, double gx, double gy, Real *state,
              Real *idiff)
{
    long c;
    for (c = 0; c < nx * ny; c++) {
        orc_gid[0] = (unsigned long)(c % nx);
        orc_gid[1] = (unsigned long)(c / nx);
        diff_step((unsigned long)nx, (unsigned long)ny, (Real)gx, (Real)gy,
                  state, idiff);
    }
}

/* cell_step over an nx x ny grid (openclsim.cl:298-367) */
void ftk_cell(long nx, long ny, double time, double dt, double pace,
              Real *state, Real *idiff, Real *inter, Real *field)
{
    long c;
    for (c = 0; c < nx * ny; c++) {
        orc_gid[0] = (unsigned long)(c % nx);
        orc_gid[1] = (unsigned long)(c / nx);
        cell_step((unsigned long)nx, (unsigned long)ny, (Real)time, (Real)dt,
                  (Real)pace, state, idiff, inter, field);
    }
}

#ifdef FTK_JUNCTION
/* diff_step_fiber_tissue over the nfy junction cells (:601-628) */
void ftk_junction(long nfx, long nfy, long ntx, long ctx, long cty, long nsf,
                  long nst, int ivf, int ivt, double gft, Real *state_f,
                  Real *state_t, Real *idiff_f, Real *idiff_t)
{
    long c;
    for (c = 0; c < nfy; c++) {
        orc_gid[0] = (unsigned long)c;
        orc_gid[1] = 0;
        diff_step_fiber_tissue(
            (unsigned long)nfx, (unsigned long)nfy, (unsigned long)ntx,
            (unsigned long)ctx, (unsigned long)cty, (unsigned long)nsf,
            (unsigned long)nst, ivf, ivt, (Real)gft, state_f, state_t,
            idiff_f, idiff_t);
    }
}
#endif
