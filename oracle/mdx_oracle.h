/*
 * mdx_oracle.h -- CPU restatement of the MDynaMix force path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this;
 * only tests, the smoke check and the CPU-baseline leg of the benchmark do.
 *
 * Parity status: pinned to the reference's own example run (its input,
 * restart file and printed output, as fixtures under tests/golden/): setup
 * numbers to the printed digits, run averages within stated bars.  The
 * reference is Fortran and no Fortran compiler exists on either machine, so
 * no bit-for-bit comparison with the original program exists; physical
 * invariants (Newton's third law, finite-difference forces, Ewald alpha
 * independence, NVE energy conservation) in tests/ pin the rest.
 *
 * The functions take the same structures as the C ABI in include/mdx_gpu.h
 * and mirror the reference routines one to one (ox_chcnb = CHCNB, ...).
 */
#ifndef MDX_ORACLE_H
#define MDX_ORACLE_H
#include "mdx_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ox_state ox_state;

int ox_open(const mdx_dims *d, const mdx_topo *t, const mdx_params *p,
            ox_state **out);
void ox_close(ox_state *st);
const char *ox_last_error(const ox_state *st);
int ox_set_threads(ox_state *st, int n);
int ox_set_params(ox_state *st, const mdx_params *p);
int ox_set_state(ox_state *st, const double *sx, const double *sy,
                 const double *sz, const double *vx, const double *vy,
                 const double *vz, const mdx_thermo *th);
int ox_get_state(ox_state *st, double *sx, double *sy, double *sz, double *vx,
                 double *vy, double *vz, mdx_thermo *th);
int ox_get_forces(ox_state *st, int which, double *fx, double *fy, double *fz);
int ox_get_bonded_averages(ox_state *st, double *br, double *be, double *ar,
                           double *ae, double *tr, double *te);

int ox_inifur(ox_state *st, int32_t *nkv);
int ox_chcnb(ox_state *st, int32_t *mbsh, int32_t *mbln);
int ox_get_lists(ox_state *st, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                 int32_t *nbl1, int32_t *nbl2, int32_t cap_l);
int ox_getcom(ox_state *st);
int ox_getkin(ox_state *st, const double *summd, double enerf_tempf, double fnop,
              double fnstr, double fnsti, double *out);
int ox_chkmom(ox_state *st, double sumasd, double *dv);
int ox_fforces(ox_state *st, int laver, mdx_scalars *out);
int ox_slforces(ox_state *st, mdx_scalars *out);
int ox_allforce(ox_state *st, mdx_scalars *out);
int ox_double(ox_state *st, int32_t nsteps, int32_t nsttot,
              mdx_step_record *rec);
int ox_double_steps(ox_state *st, int32_t nsteps, int32_t mstep0,
                    mdx_step_record *rec);
int ox_sultan(ox_state *st, int32_t nsteps, int32_t nsttot,
              mdx_step_record *rec);
int ox_sultan_steps(ox_state *st, int32_t nsteps, int32_t mstep0,
                    mdx_step_record *rec);
int ox_set_lambda(ox_state *st, double ec, double pw1, double pw2, double bee);
int ox_set_pullback(ox_state *st, const mdx_pullback *pb);
int ox_ee_delta(ox_state *st, double ec_old, double ec_new, double pw1, double pw2,
                double bee, double *out);
/* PIMD over nbeads bead states (pimd.f:18-444); thermo: THERMO(NSTOT, JNH)
 * column-major, in and out; prologue: run the preparation 1.2 first. */
int ox_pimd_steps(ox_state *const *beads, const mdx_pimd_params *pp, double *thermo,
                  int32_t nsteps, int32_t mstep0, int prologue, mdx_pimd_record *rec);

#ifdef __cplusplus
}
#endif
#endif
