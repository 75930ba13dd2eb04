/*
 * suli_oracle.h -- CPU oracle for the SuLi-IC per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-faithful FP64 restatement of the
 * reference Fortran routines (the SuLi-IC .f90 files), used by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's cpu_baseline /
 * --impl reference arm.  The product (suli_gb300, libsuli_gpu.so) never links,
 * loads or calls it.
 *
 * Parity status: pinned against outputs of the reference itself.  The
 * reference ships no tests, golden vectors or fixtures, and no Fortran
 * compiler exists in this build environment; tests/golden/f90sub.py runs the
 * Fortran 90 subset of the reference's hot-path files by translating it to
 * Python (IEEE binary64, the reference's evaluation order, glibc's libm), and
 * tests/golden/make_golden.py records 18 small cases after whole time steps
 * of the reference's own routines (dam break with all five time schemes,
 * Smagorinsky and k-equation LES/DES, the IPA, surface tension, both
 * sponges, the image-point IBM, SuLi-ICdz's variable z spacing, Stokes
 * I/II/V waves through the inflow), three RK stages routine by routine from
 * random states, and PRTSCR's field records; every subscript is
 * bounds-checked, so no vector rests on memory the Fortran leaves undefined
 * (the inflow fill's one read below its array takes face 1, as here).  tests/test_golden_reference.py holds this
 * oracle to those fixtures: every field bit for bit.  Analytic known-answer
 * tests (WENO5 exactness on polynomials, manufactured-solution convergence,
 * divergence-free projection, still water at rest, conservation) add to it,
 * see tests/test_oracle_*.py.
 *
 * Arrays use the reference's layout: column-major, i fastest, with the same
 * lower bounds as the Fortran allocations (0_modules.f90).
 */
#ifndef SULI_ORACLE_H
#define SULI_ORACLE_H

#include "../include/suli_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_case or_case;

or_case *or_create(const suli_params *p);
void     or_destroy(or_case *c);

/* Pointer to the case's array for a suli_field id (reference layout,
 * double except id_ibm* which are int32).  lo/hi receive the bounds. */
void    *or_field(or_case *c, int field, int lo[3], int hi[3]);
int      or_set_scalar(or_case *c, int scalar, double v);
double   or_get_scalar(or_case *c, int scalar);

/* Initial conditions (2_iniciais.f90:127-274, 14_level_set.f90:10-200). */
void or_level_set_ini(or_case *c, int tipo, double ampl, double lambdax,
                      double lambday, double prof, double m);
void or_heaviside_init(or_case *c);           /* heaviside + vol_ini */
void or_iniciais_velocity(or_case *c);        /* v=w=prd=0, u=uinicial, b?? planes */
void or_mms_init(or_case *c);                 /* 13_mms.f90:39-114 (mms_t=1) */
void or_termo_fonte1(or_case *c);             /* 13_mms.f90:820-1065 */
void or_obstaculo_cylinder(or_case *c, double xc, double yc, double radius);
void or_ibm_setup(or_case *c);                /* reinit obstacle ls, ibm_posicoes, 3_contorno.f90:991-1004 */

/* Hot-path routines (one per reference subroutine). */
void or_level_set(or_case *c);                /* 14_level_set.f90:204-273 */
void or_contorno(or_case *c, int nlock);      /* 3_contorno.f90:11-662 */
void or_visco(or_case *c);                    /* 5_viscosidade.f90:11-157 */
void or_convdiff(or_case *c);                 /* 6_convdiff.f90:14-167 */
void or_complementos(or_case *c);             /* 11_diversos.f90:355-450 */
void or_tempo(or_case *c);                    /* 11_diversos.f90:10-296 */
int  or_graddin(or_case *c);                  /* 9_grad.f90:10-663, returns iterations */
void or_posdin(or_case *c);                   /* 10_pos.f90:1-99 */
void or_exp_press(or_case *c);                /* 11_diversos.f90:455-495 (t_press = 2) */
void or_contorno_les(or_case *c);             /* 3_contorno.f90:666-790 */
void or_boundary_waves(or_case *c);           /* 3_contorno.f90:1189-1319 */
double or_conmassa(or_case *c);               /* 4_plot.f90:386-394, returns max|div| */
int  or_prtscr_write(or_case *c, const char *path, int t_plot); /* 4_plot.f90:547-615 */
void or_mms_error(or_case *c, double err[4]); /* 13_mms.f90:391-451 */
void or_set_stage(or_case *c, int tt);        /* 1_principal.f90:86-87 */
void or_step(or_case *c);                     /* 1_principal.f90:69-124 */

/* Low-level pieces exposed for unit known-answer tests. */
void or_weno_line(const double *a, long stride, int n, double h, int ihs,
                  double *dp, double *dn);    /* 8_derivadas.f90:675-811 */

/* Diagnostics of the last step. */
void or_diag(or_case *c, suli_diag *d);

/* Replay of data-dependent iteration counts (parity runs): when >= 0 the
 * next graddin calls run exactly this many CG iterations / the next reinit
 * exactly this many iterations.  -1 = free running (reference rules). */
void or_set_replay(or_case *c, const int cg_iters[3], int reinit_iters);

void or_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
