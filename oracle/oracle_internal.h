/* oracle_internal.h -- helpers shared by the oracle's translation units
   (TEST INFRASTRUCTURE ONLY). */
#ifndef CAP_ORACLE_INTERNAL_H
#define CAP_ORACLE_INTERNAL_H

/* 0-based storage index of the reference's ijk = lk(k)+li(i)+j */
#define IXK(i, j, k) (s->lk[(k)] + s->li[(i)] + (j) - 1)

/* modules_allocatable.f90:39-40: small/great are default-real (single
   precision) literals assigned to real(dp) parameters. */
#define SMALL ((double)1e-30f)
#define GREAT ((double)1e+30f)

static inline double dmin(double a, double b) { return a < b ? a : b; }
static inline double dmax(double a, double b) { return a > b ? a : b; }

int cap_solve_dispatch(cap_state* s, int solver, int fi, int ifi, cappgpu_solve_report* rep);

#endif
