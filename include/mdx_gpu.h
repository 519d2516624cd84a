/*
 * mdx_gpu.h -- C ABI of the GB300 (sm_103a) force path for MDynaMix.
 *
 * The library replaces the per-step force path of MDynaMix v5.3 (Fortran).
 * The Fortran driver keeps its COMMON blocks, its input, its output and its
 * step loop; at the points below it calls these functions instead of the
 * Fortran routines.  Every entry point states the reference routine it
 * replaces (file:line within the MDynaMix source tree).
 *
 *   mdx_chcnb        <- CHCNB(LRDF)            forces.f:1813-2205
 *   mdx_fforces      <- FFORCES(LAVER)         forces.f:36-51
 *   mdx_slforces     <- SLFORCES               forces.f:55-73
 *   mdx_allforce     <- ALLFORCE               forces.f:77-100
 *   mdx_getcom       <- GETCOM                 service.f:463-563
 *   mdx_getkin       <- GETKIN (no GETROT)     service.f:611-735
 *   mdx_chkmom       <- CHKMOM                 service.f:1081-1125
 *   mdx_double       <- DOUBLE (whole body)    mdstep.f:281-530
 *   mdx_double_steps <- DOUBLE loop 2.3 only   mdstep.f:324-436
 *   mdx_sultan       <- SULTAN (whole body)    mdstep.f:29-260
 *   mdx_sultan_steps <- SULTAN loop 1.3 only   mdstep.f:83-162
 *   mdx_set_lambda   <- RECINT                 mdee.f:86-140
 *   mdx_inifur       <- INIFUR                 forces.f:1356-1449
 *
 * Conventions
 *  - Plain C: pointers and sizes only.  All arrays are copied in at the call;
 *    no host pointer is retained after a call returns.
 *  - Index arrays are the Fortran ones, 1-based, exactly as they sit in the
 *    COMMON blocks (ITYPE, NNUM, NSITE, INBB, IBI, ...).  Two-dimensional
 *    Fortran arrays are passed column-major with their leading dimension.
 *  - Coordinates are in Angstrom; every other quantity is in the reference's
 *    internal units (setup.f:95-113), i.e. the tables the Fortran has already
 *    converted (A6LJ, B12LJ, FB, COULF, MASSDI, ...).
 *  - Velocities are the reference's VX/VY/VZ, which hold momenta
 *    (kinetic energy = sum VX**2*MASSDI/2, service.f:50-60).
 *  - Return value: MDX_OK (0) or an MDX_ERR_* code; mdx_last_error() gives
 *    the message.  The Fortran shim turns a nonzero code into a message and
 *    CALL FINAL, which is what the reference does on the same conditions.
 *  - One context = one system on one CUDA stream, single host thread.
 */
#ifndef MDX_GPU_H
#define MDX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDX_NTPS 10                                  /* dimpar.h:26  NTPS  */
#define MDX_NTPP ((MDX_NTPS * (MDX_NTPS + 1)) / 2 + 1) /* dimpar.h:50  NTPP  */

/* return codes */
enum {
  MDX_OK = 0,
  MDX_ERR_ARG = 1,            /* bad argument or inconsistent sizes           */
  MDX_ERR_CUDA = 2,           /* CUDA runtime error                           */
  MDX_ERR_LIST_OVERFLOW = 3,  /* neighbour list capacity (forces.f:2188-2194)  */
  MDX_ERR_SHAKE = 4,          /* SHAKE did not converge in MAXIT (mdstep.f:1264)*/
  MDX_ERR_NAN = 5,            /* non-finite force, energy or coordinate        */
  MDX_ERR_TIMEOUT = 6,        /* a bounded device wait ran out                 */
  MDX_ERR_STATE = 7,          /* call made before what it depends on           */
  MDX_ERR_NOMEM = 8,          /* device allocation failed                      */
  MDX_ERR_KVEC = 9,           /* more k-vectors than NKVM (forces.f:1414-1419) */
  MDX_ERR_UNSUPPORTED = 10    /* option outside the built path                 */
};

/* precision of the force path */
enum { MDX_FP64 = 0, MDX_MIXED = 1 };

/* Sizes fixed for the life of a context (the dimpar.h role). */
typedef struct {
  int32_t nstot;      /* NSTOT  atoms                                  */
  int32_t nop;        /* NOP    molecules                              */
  int32_t ntypes;     /* NTYPES molecule types (<= MDX_NTPS)           */
  int32_t nsites;     /* NSITES sites, summed over types               */
  int32_t nnbt;       /* NNBT   non-bonded (LJ) types                  */
  int32_t nrbb;       /* NRBB   bond records over all types            */
  int32_t nraa;       /* NRAA   angle records                          */
  int32_t nrtt;       /* NRTT   torsion records                        */
  int32_t nrbt;       /* NRBT   bond instances (all molecules)         */
  int32_t nrat;       /* NRAT   angle instances                        */
  int32_t nrrt;       /* NRRT   torsion instances                      */
  int32_t nbdmax;     /* NBDMAX columns of INBB                        */
  int32_t cap_short;  /* short-list pairs owned per atom (NBSMX role)  */
  int32_t cap_long;   /* long-list pairs owned per atom (NBLMX role)   */
  int32_t nkv_max;    /* NKVM   maximum k-vectors                      */
  int32_t precision;  /* MDX_FP64 or MDX_MIXED                         */
} mdx_dims;

/* Topology and tables, as produced by IUNITS/BNDLST (setup.f:27-888). */
typedef struct {
  /* per atom, length nstot (/ADDREFS/, /SITSITM/) */
  const int32_t *itype;   /* ITYPE atom -> molecule type  */
  const int32_t *nnum;    /* NNUM  atom -> molecule       */
  const int32_t *nsite;   /* NSITE atom -> site           */
  const double *massdi;   /* MASSDI inverse mass          */
  const double *q;        /* Q charge (EE-scaled)         */
  /* per site, length nsites (/SITTES/) */
  const double *charge;   /* CHARGE                       */
  const double *mass;     /* MASS (atomic units)          */
  const int32_t *inbt;    /* INBT site -> LJ type         */
  /* per molecule type, length ntypes (/MOLTYP/, /SOMMOL/, /MDEEI/) */
  const int32_t *nspec, *nsits;
  const int32_t *isadr;   /* ISADR(ityp)  sites before type  */
  const int32_t *isaddr;  /* ISADDR(ityp) atoms before type  */
  const int32_t *iaddr;   /* IADDR(ityp)  molecules before   */
  const int32_t *ipot;    /* IPOT special water potential    */
  const int32_t *nrb;     /* NRB bonds per molecule          */
  const int32_t *iadb;    /* IADB first bond record of type  */
  const int32_t *ishejk;  /* ISHEJK constrain this type      */
  const int32_t *iee;     /* IEE 0 = expanded-ensemble type  */
  const int32_t *lmove;   /* LMOVE (0/1)                     */
  const double *c14el, *c14lj, *summas;
  /* LJ tables NNBT x NNBT, column-major, leading dimension ld_lj (/SITTES/) */
  const double *a6lj, *b12lj, *a6lj0, *b12lj0, *a6_14, *b12_14;
  int32_t ld_lj;
  /* MDX(ityp,jtyp) type-pair index, column-major, leading dimension ld_mdx */
  const int32_t *mdx;
  int32_t ld_mdx;
  /* exclusions from BNDLST: NNBB(nstot), INBB(ld_inbb, nbdmax) signed */
  const int32_t *nnbb;
  const int32_t *inbb;
  int32_t ld_inbb;
  /* bond records, length nrbb (/BONBON/) */
  const int32_t *ib, *jb, *id;
  const double *rb, *fb, *db, *ro;
  /* bond instances, length nrbt */
  const int32_t *ibi, *jbj, *ibuk;
  /* angle records, length nraa, and instances, length nrat (/ANGANG/) */
  const double *ra, *fa;
  const int32_t *iai, *jaj, *kak, *iauk;
  /* torsion records, length nrtt, and instances, length nrrt (/TORTOR/) */
  const int32_t *itors, *nmul;
  const double *ft, *rt, *ft1, *ft2, *ft3, *ft4, *ft5;
  const int32_t *iti, *jtj, *ktk, *ltl, *ituk;
  /* per bond record (length nrbb): 1 if SHEJK holds it as a constraint.
   * NULL gives the reference's rule, every record with ID != 2
   * (mdstep.f:1135); a flag per record allows e.g. bonds to hydrogen only,
   * which the reference cannot express (its ID = 2 also drops the pair
   * from the exclusions, setup.f:787). */
  const int32_t *lcon;
} mdx_topo;

/* Run parameters (/SIZES/, /ENERGY/, /NVTNPT/, main.f:380-450, 729-812). */
typedef struct {
  double boxl, boyl, bozl;   /* box lengths (Angstrom)                   */
  int32_t icell;             /* ICELL 0 rect, 1 truncated oct, 2 hex
                                (both paths); BOYL = BOXL cos30 for hex,
                                BOYL = BOZL = BOXL for oct, as RECLEN
                                leaves them; not with a Verlet skin      */
  int32_t lmnbl;             /* reaction field instead of Ewald          */
  double coulf;              /* COULF                                    */
  double alphad;             /* ALPHAD Ewald alpha (1/Angstrom)          */
  double fexp;               /* FEXP  (B): |k|^2 <= 4 alpha^2 B          */
  double rcut;               /* RCUT (RCUTT; RSSQ = RCUTT**2)            */
  double rshort;             /* SHORT                                    */
  double rskin;              /* 0: the reference's list (CHCNB every ICHNB
                                long steps, pairs evaluated as listed);
                                > 0: Verlet-skin mode, not in the reference:
                                list radius RCUT + rskin, pairs beyond RCUT
                                skipped at evaluation, rebuilt once an atom
                                has moved rskin / 2 (ICHNB unused); constant
                                volume only                               */
  double rff, rff2;          /* reaction-field constants                 */
  double tstep, tsteb;       /* TSTEP, TSTEB                             */
  int32_t nfreq;             /* NFREQ short steps per long step          */
  int32_t ichnb;             /* ICHNB list refresh period (long steps)   */
  int32_t lshejk;            /* SHAKE on                                 */
  int32_t maxit;             /* SHAKE MAXIT (2000 in mdstep.f:1110)      */
  double toler, bdtol;       /* TOLER, BDTOL                             */
  int32_t lnvt, lnpt, lsep, lsctd, lp_xy, lsclt, lscft;
  double trtemp, tdelt;      /* TRTEMP, TDELT                            */
  double trpres, trpresx, trpresy, trpresz;
  double dqt, dqp, rtp;      /* thermostat/barostat constants (main.f)   */
  double fnst, fnop;         /* FNST degrees of freedom, FNOP            */
  double ftscl, ftimes;      /* FTSCL = 1 / Cut_forces level (main.f:850),
                                FTIMES                                  */
  double convet;             /* CONVET (setup.f:119)                     */
  double unitp;              /* UNITP                                    */
  double efact;              /* EFACT = 1.D3/AVSNO/UNITE (setup.f:395)   */
  double tfact[MDX_NTPS];    /* TFACT per type                           */
  double tridm_coef;         /* NOP*BOLTZ*1e-5/UNITL**3                  */
  double tridee_coef;        /* (1-EC(ME))*NDEL*BOLTZ*TRTEMP*1e-5/UNITL**3 */
  double epd, vird;          /* LJ tail corrections EPD, VIRD (ELRCLJ)   */
  double chktf;              /* temperature watchdog factor (0 = off)    */
  int32_t lmdee;             /* expanded ensemble active                 */
  double raex;               /* RAEX soft-core shift                     */
  double ec_me;              /* EC(ME) for INIFUR's self-energy          */
  int32_t ntyp1;             /* NTYPES+1                                 */
  int32_t molint;            /* MOLINT = type pairs + 1                  */
} mdx_params;

/* Energies and virials of one force evaluation (/ENERGY/, /VIRRR/, /SOMMOL/). */
typedef struct {
  double pe1, pels1, pe2, pels2, spe, pint, qpe;
  double vir1, vir2, virb, virx, viry, virz, virfx, virfy, virfz;
  double wirs, wirss;
  double pote1[MDX_NTPP], potl1[MDX_NTPP];
  double pes141[MDX_NTPS], psr141[MDX_NTPS], spee[MDX_NTPS];
  int32_t mbsh, mbln, nkv;   /* list sizes and k-vectors in use           */
  int32_t lscfl;             /* SCLFRC cut forces in this evaluation      */
} mdx_scalars;

/* Thermostat/barostat state and derived quantities (/NVTNPT/, GETEMP, SCALING). */
typedef struct {
  double sc, scl, sclx, scly, sclz;
  double scm[MDX_NTPS];
  double eabs;
  double boxl, boyl, bozl, vol;
  /* outputs */
  double tke, temp, tempr[MDX_NTPS + 4], ekin[MDX_NTPS + 4];
  double virkx, virky, virkz;
  double vira[3], viran[3];
  double tryck, tryckm, tryckx, trycky, tryckz;
  int32_t shake_iter_max;    /* largest SHAKE iteration count seen        */
  int32_t shake_fail;        /* molecules past MAXIT; the reference prints
                                a message and goes on (mdstep.f:1264-1269) */
  int32_t nscale;            /* forced velocity rescalings (NRTSC)        */
  int32_t npt_fail;          /* NPT "too strong fluctuations" count (ISKK) */
  int32_t list_builds;       /* CHCNB builds done (counted on the device)  */
  int32_t reserved;
} mdx_thermo;

/* One record per long step, filled on the device and copied back once. */
typedef struct {
  int32_t mstep;
  int32_t mbsh, mbln;
  int32_t shake_iter;
  double pe1, pels1, pe2, pels2, spe, pint;
  double vir1, vir2, virb, virx, viry, virz, virfx, virfy, virfz, wirs, wirss;
  double tke, temp, sc, scl, tryck, tryckm;
  double boxl, boyl, bozl, vol;
  double eabs;
} mdx_step_record;

typedef struct mdx_ctx mdx_ctx;

/* lifetime */
int mdx_open(const mdx_dims *dims, mdx_ctx **out);
int mdx_close(mdx_ctx *ctx);
const char *mdx_last_error(const mdx_ctx *ctx);
const char *mdx_strerror(int code);
int mdx_version(void);

/* data in and out */
int mdx_upload_topology(mdx_ctx *ctx, const mdx_topo *topo);
int mdx_set_params(mdx_ctx *ctx, const mdx_params *par);
int mdx_upload_state(mdx_ctx *ctx, const double *sx, const double *sy,
                     const double *sz, const double *vx, const double *vy,
                     const double *vz, const mdx_thermo *th);
int mdx_download_state(mdx_ctx *ctx, double *sx, double *sy, double *sz,
                       double *vx, double *vy, double *vz, mdx_thermo *th);
/* Asynchronous copy of the state for restart dumps and trajectory frames
 * written off the step loop (RESTRT(2) restart.f:308-420 and TRACE
 * restart.f:425-598 read SX/VX on the host; the reference stops its step
 * loop to write them).  mdx_snapshot queues, on the context's stream and
 * after the work already queued there, the copy of positions, momenta and
 * (th != NULL) the thermostat/box state into the given host buffers, and
 * returns at once; use page-locked buffers (a copy into pageable memory
 * waits for the stream).  mdx_snapshot_wait(slot) blocks until that copy has
 * landed and may be called from another host thread.  Slots 0 ..
 * MDX_SNAPSHOT_SLOTS-1 let several snapshots be in flight; a slot's buffers
 * must not be reused before its wait returns.  The first call allocates a
 * device staging buffer and waits for the stream once. */
#define MDX_SNAPSHOT_SLOTS 8
int mdx_snapshot(mdx_ctx *ctx, int32_t slot, double *sx, double *sy, double *sz,
                 double *vx, double *vy, double *vz, mdx_thermo *th);
int mdx_snapshot_wait(mdx_ctx *ctx, int32_t slot);
/* which: 1 = H (fast), 2 = G (slow), 3 = F = G + H */
int mdx_download_forces(mdx_ctx *ctx, int which, double *fx, double *fy,
                        double *fz);

/* routines of forces.f / service.f */
int mdx_inifur(mdx_ctx *ctx, int32_t *nkv);
int mdx_chcnb(mdx_ctx *ctx, int32_t *mbsh, int32_t *mbln);
/* The lists of the last mdx_chcnb in the reference's layout and order:
 * NBS1/NBS2 (short, 1-4 pairs with negative first index) and NBL1/NBL2. */
int mdx_get_lists(mdx_ctx *ctx, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                  int32_t *nbl1, int32_t *nbl2, int32_t cap_l);
int mdx_getcom(mdx_ctx *ctx);
/* GETKIN: translational, rotational and internal kinetic energies and
 * temperatures from the current momenta and the molecule-relative site
 * vectors of the last GETCOM.  summd[t] = SUMMAS(t) / (AVSNO 1000 UNITM
 * NBEADS) for the ntypes types; enerf_tempf = ENERF TEMPF; fnop, fnstr,
 * fnsti = FNOP, FNSTR, FNSTI (main.f:297-346).  The molecular orientation
 * analysis (GETROT, LMOL1/LMOL2) is not part of it. */
typedef struct mdx_kin {
  double ektr, ekrot, ekint, tke; /* EKTR, EKROT, EKINT, TKE */
  double ttr, trot, tint;         /* TTR, TROT, TINT */
} mdx_kin;
int mdx_getkin(mdx_ctx *ctx, const double *summd, double enerf_tempf, double fnop,
               double fnstr, double fnsti, mdx_kin *out);
/* CHKMOM: removes the total momentum (sumasd = TOTMAS / UNITM) and updates
 * the temperature as GETEMP; dv (optional) receives the removed DVX, DVY,
 * DVZ. */
int mdx_chkmom(mdx_ctx *ctx, double sumasd, double *dv);
int mdx_fforces(mdx_ctx *ctx, int laver, mdx_scalars *out);
int mdx_slforces(mdx_ctx *ctx, mdx_scalars *out);
int mdx_allforce(mdx_ctx *ctx, mdx_scalars *out);

/* integrators of mdstep.f; rec (optional) receives nsteps records */
int mdx_double(mdx_ctx *ctx, int32_t nsteps, int32_t nsttot,
               mdx_step_record *rec);
int mdx_double_steps(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0,
                     mdx_step_record *rec);
int mdx_sultan(mdx_ctx *ctx, int32_t nsteps, int32_t nsttot,
               mdx_step_record *rec);
int mdx_sultan_steps(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0,
                     mdx_step_record *rec);

/* Asynchronous DOUBLE for a host loop that drives many contexts at once
 * (no counterpart in the reference, whose step loop is synchronous).
 * mdx_double_enqueue puts nsteps long steps (mdstep.f:324-436) on the
 * context's stream, optionally preceded by DOUBLE's prologue (CHCNB, GETCOM,
 * SLFORCES, FFORCES; mdstep.f:296-310), and returns without waiting; steps
 * are replayed from captured CUDA graphs, so constant volume and timers off
 * are required (MDX_ERR_STATE otherwise).  mdx_poll sets *done = 1 once all
 * enqueued work has finished and then returns its error status, exactly as
 * mdx_double would; *done = 0 while work is in flight.  mdx_device_memory
 * reports the device's free and total bytes (cudaMemGetInfo), for admission
 * by memory budget. */
int mdx_double_enqueue(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0, int32_t prologue);
int mdx_poll(mdx_ctx *ctx, int32_t *done);
int mdx_device_memory(size_t *free_bytes, size_t *total_bytes);
/* Diagnostic: bytes in use and reserved in the current device's default
 * memory pool, from which contexts allocate (cudaMallocAsync). */
int mdx_pool_usage(size_t *used_bytes, size_t *reserved_bytes);
/* Which kernels the context runs, for reports next to measured numbers (no
 * counterpart in the reference).  Valid once the k-set exists.
 *  ewald_force_pass: 0 FP64 CUDA cores; 1 FP32 CUDA cores; 2 TF32 tensor
 *                    cores, three products per operand pair.
 *  ewald_sfac_pass:  0 FP64 per slice, slices summed in FP64; 1 FP32 FMAs
 *                    per slice, slices summed in FP64; 2 TF32 tensor cores
 *                    with FP32 partials of 1024 atoms summed in FP64.
 *  sfac_ordered:     1 when slice partials are summed in slice order (the
 *                    reciprocal sums are then reproducible run to run).
 *  list_mode:        0 the reference's (CHCNB every ICHNB long steps);
 *                    1 Verlet skin. */
typedef struct {
  int32_t precision, ewald_force_pass, ewald_sfac_pass, sfac_slices;
  int32_t sfac_ordered, list_mode, graphs, nkv;
} mdx_path_info;
int mdx_get_path_info(const mdx_ctx *ctx, mdx_path_info *out);

/* Work split of the mixed pair sweeps: threads per owner atom of the short
 * rows (tpo_short: 2, 4 or 8) and of the long rows (tpo_long: 4, 8, 16 or 32).
 * No counterpart in the reference (a launch-shape choice of this library).
 * By default a context takes the choice of the tuning table built into the
 * library (written by mdynamix_gb300/autotune.py from timings of each split
 * on a GB300, keyed by system size and mean row length), fixed at its first
 * pair sweep from the sizes alone, so equal systems always run the same
 * split.  The split changes the FP32 lane partials before the fixed-point
 * sums, so forces differ between splits at the mixed path's rounding level,
 * not beyond.  mdx_set_tuning overrides it (NULL: back to the table) and
 * drops the captured step graphs; set it before a PIMD ensemble is opened
 * on the context.  source: 1 table, 2 mdx_set_tuning. */
typedef struct {
  int32_t tpo_short, tpo_long, source, reserved;
} mdx_tuning;
int mdx_set_tuning(mdx_ctx *ctx, const mdx_tuning *t);
int mdx_get_tuning(mdx_ctx *ctx, mdx_tuning *out);
/* Diagnostic: the CUDA runtime error recorded for the calling thread and not
 * yet consumed (0 = none), without clearing it. */
int mdx_pending_cuda_error(void);

/* SLFORCES without device allocation.  No counterpart in the reference (its
 * FURIR uses static COMMON arrays; this library's mdx_slforces keeps the S(k)
 * partial sums in a device buffer it allocates with the k-set).  For callers
 * that must not allocate device memory during a run: a host loop that has
 * handed its HBM budget to many resident contexts and cannot have a call
 * fail or fragment memory half way, or one that cannot afford cudaMalloc's /
 * cudaFree's implicit device-wide synchronisation, which stalls every other
 * stream on the GPU.  Same kernels and results as mdx_slforces, with the S(k)
 * scratch in one static device array of MDX_SK_STATIC_BYTES per device.
 * Returns MDX_ERR_UNSUPPORTED when slices x k-vectors x 16 bytes exceed it,
 * MDX_ERR_STATE when the k-set is not built yet or the box left its 5 %
 * window (a new k-set allocates: call mdx_inifur), or when timers are on.
 * The first call on a device sets up the scratch address; make it before any
 * stream capture.  Under CUDA's lazy module loading that first call also
 * loads the module that holds the array, so it reserves the 4 MiB then and
 * can fail with MDX_ERR_CUDA when the device is full; later calls cannot.
 * The address is cached per device for the process: do not cudaDeviceReset
 * between calls.  With the mixed path's tensor-core S(k) pass on
 * (MDX_EWALD_TC=2) the pass needs no slice scratch and the size limit does
 * not apply.  Calls whose kernels overlap on the device (other
 * contexts, other streams or threads) share the scratch and race: serialise
 * them. */
#define MDX_SK_STATIC_BYTES (4u << 20)
int mdx_slforces_static(mdx_ctx *ctx, mdx_scalars *out);

/* GETAVR's per-term statistics (aver.f:45-100) from the device.  The bonded
 * routines form, per bond / angle / torsion record, the average over the
 * type's molecules of its length (angle, dihedral) and energy -- BR/BE,
 * AR/AE, TR/TE (forces.f:181-182, 272-273, 446-447) -- at every FFORCES
 * with LAVER here.  mdx_get_bonded_averages returns those of the last such
 * evaluation (NRBB, NRBB, NRAA, NRAA, NRTT, NRTT values; any pointer may be
 * NULL; internal units, angles in radians).  With mdx_set_averaging(ctx, 1)
 * every long step of DOUBLE / SULTAN evaluates its last fast forces with
 * LAVER and adds the values and their squares to device sums;
 * mdx_get_bonded_sums copies them out (1 + 4 (NRBB + NRAA + NRTT) doubles:
 * the sample count, the sums of BR, BE, AR, AE, TR, TE back to back, then
 * the sums of their squares in the same order) and, with clear != 0,
 * restarts them -- the host keeps no per-step work at IAVER = 1. */
int mdx_get_bonded_averages(mdx_ctx *ctx, double *br, double *be, double *ar, double *ae,
                            double *tr, double *te);
int mdx_set_averaging(mdx_ctx *ctx, int on);
int mdx_get_bonded_sums(mdx_ctx *ctx, double *sums, int32_t clear);

/* PULLBACK (forces.f:1756-1799): what SLFORCES and ALLFORCE add to the slow
 * forces G after the pair and Ewald terms and before SCLFRC -- a constant
 * drag on the atoms of chosen types (LDRAG: GZ += MASSD FDRAG), harmonic
 * wells that hold chosen atoms near reference positions (LRR: G -= RLR
 * (S - S_ref), no minimum image, as the reference), and an external field
 * along z (IEXT = 1: GZ += Q EXAMPL cos(EXFREQ FULTIM / (2 PI)), FULTIM =
 * TIM + NSTEP DT).  NSTEP counts long steps on the device: nstep at the
 * call, one more at the start of every DOUBLE / SULTAN long step.  pb =
 * NULL switches it off.  Arrays are copied in. */
typedef struct {
  int32_t ldrag;                 /* LDRAG                                   */
  int32_t ldragt[MDX_NTPS];      /* LDRAGT per molecule type                */
  double fdrag[MDX_NTPS];        /* FDRAG per type (internal units)          */
  int32_t npull;                 /* NPULL atoms in wells (LRR when > 0)      */
  const int32_t *inpl;           /* INPL: their atom numbers, 1-based        */
  const double *xpl, *ypl, *zpl; /* XPL, YPL, ZPL: the wells' centres (A)    */
  double rlr;                    /* RLR spring constant (internal units)     */
  int32_t iext;                  /* IEXT: 1 = external field along z         */
  double exampl, exfreq;         /* EXAMPL, EXFREQ                           */
  double tim, dt;                /* TIM and DT (seconds)                     */
  int32_t nstep;                 /* NSTEP of the next force evaluation       */
} mdx_pullback;
int mdx_set_pullback(mdx_ctx *ctx, const mdx_pullback *pb);

/* expanded-ensemble scaling (RECINT) */
int mdx_set_lambda(mdx_ctx *ctx, double ec, double pw1, double pw2,
                   double bee);
/* Energy differences for an expanded-ensemble move from the current
 * subensemble (coupling ec_old = EC(ME), the one the last mdx_set_lambda
 * set) to ec_new = EC(ME1), at the current positions and lists:
 * out[0..3] = EFN, EFO (DIFFUR mdee.f:265-376: reciprocal Ewald sum, self
 * and intramolecular Ewald terms of the new and the old charges) and EEN,
 * EEO (DIFEN mdee.f:379-536: LJ and real-space Ewald of the listed pairs
 * between an EE molecule and any other molecule), internal energy units.
 * CHENS (mdee.f:142-262) forms DE = (EEN - EEO + EFN - EFO + EELRC(ME1) -
 * EELRC(ME)) BETA - EE(ME1) + EE(ME) on the host, draws the Metropolis
 * decision and, on acceptance, calls mdx_set_lambda(ec_new).  The
 * reciprocal part re-forms S(k) at the current positions (FURIR's first
 * half); forces are untouched. */
int mdx_ee_delta(mdx_ctx *ctx, double ec_old, double ec_new, double pw1, double pw2,
                 double bee, double *out);

/* Path-integral MD (pimd.f): NBEADS contexts, one per bead replica of the
 * same system (same topology and parameters, states uploaded), advanced
 * together.  The reference runs one bead per MPI rank (input.f:643-659) and
 * couples them every short step by ring springs (PIFORCES, pimd.f:321-395;
 * neighbour-bead coordinates travel as REAL*4, pimd.f:450-486, and are used
 * rounded to single precision here too) and by per-atom Nose-Hoover chains
 * on the bead kinetic energy summed over beads (BEADNOSE, pimd.f:402-444);
 * forces of each bead are divided by NBEADS.  Here all beads stay on one
 * GPU; each long step is one CUDA graph whose per-bead work runs on the
 * beads' own streams concurrently, joined for the two cross-bead kernels.
 * Bead thermostats only (PI_thermo): a bead context with LNVT or LNPT set is
 * rejected (MDX_ERR_UNSUPPORTED). */
typedef struct {
  int32_t nbeads;   /* NBEADS (PIMD keyword)                          */
  int32_t jnh;      /* JNH bead thermostats per atom (PI_thermo)       */
  double beadfac;   /* BEADFAC, setup.f:696                            */
  double conveq;    /* CONVEQ,  setup.f:700                            */
  double dqqt;      /* DQQT,    main.f:413                             */
  double fnh;       /* FNH,     main.f:415                             */
} mdx_pimd_params;

/* One record per long step of the bead ensemble (pimd.f:225-241 quantities). */
typedef struct {
  int32_t mstep;
  double qek;       /* QEK = QEKS/NFREQ: ring-spring energy (pimd.f:229)  */
  double virpi;     /* VIRPI summed over beads                           */
  double pe;        /* PE1+PE2+PELS1+PELS2+SPE+PINT summed over beads     */
  double tke;       /* TKE summed over beads                             */
  double temp;      /* TEMP averaged over beads                          */
} mdx_pimd_record;

typedef struct mdx_pimd mdx_pimd;
int mdx_pimd_open(mdx_ctx *const *beads, const mdx_pimd_params *par, mdx_pimd **out);
int mdx_pimd_close(mdx_pimd *pi);
/* PIMD (pimd.f:18-316): the preparation 1.2 (CHCNB, GETCOM, SLFORCES,
 * FFORCES, /NBEADS, PIFORCES) then nsteps long steps; records optional. */
int mdx_pimd_run(mdx_pimd *pi, int32_t nsteps, int32_t nsttot, mdx_pimd_record *rec);
/* nsteps more long steps without the preparation. */
int mdx_pimd_steps(mdx_pimd *pi, int32_t nsteps, int32_t mstep0, mdx_pimd_record *rec);
/* The stream the bead ensemble's steps run on (for timing with events). */
void *mdx_pimd_stream(mdx_pimd *pi);
/* THERMO(NSTOT, JNH), column-major, in and out. */
int mdx_pimd_get_thermo(mdx_pimd *pi, double *thermo);
int mdx_pimd_set_thermo(mdx_pimd *pi, const double *thermo);

/* measurement helpers: the stream the context launches on, and a count of
 * the kernels it has launched since open */
void *mdx_stream(mdx_ctx *ctx);
int64_t mdx_launch_count(const mdx_ctx *ctx);
int mdx_sync(mdx_ctx *ctx);

/* Per-routine device timers, the GPU counterpart of the reference's CPU time
 * table (/TIMESZ/ in common_inc.f:102-103, printed by GETAVR, aver.f:284-297).
 * When on, CUDA events bracket each kernel group on the context's stream;
 * mdx_get_timers synchronises, returns accumulated milliseconds and launch
 * counts per group (arrays of MDX_NTIMERS) and clears them. */
enum {
  MDX_T_LIST = 0,     /* CHCNB                       (TIMEV) */
  MDX_T_PAIR_SHORT,   /* LOCALF                      (TIMES) */
  MDX_T_PAIR_LONG,    /* FORCES                      (TIMEL) */
  MDX_T_EW_TABLES,    /* FURIR phase tables          (TIMEF) */
  MDX_T_EW_SFAC,      /* FURIR structure factors     (TIMEF) */
  MDX_T_EW_KTERMS,    /* FURIR per-k energy/virial   (TIMEF) */
  MDX_T_EW_FORCE,     /* FURIR forces                (TIMEF) */
  MDX_T_ETERMS,       /* ETERMS                      (TIMEE) */
  MDX_T_BONDED,       /* GETBND/GETANG/GETTRS/STRBND (TIMEB..) */
  MDX_T_MOVE,         /* kicks, drift, GETCOM, SHAKE, SCALING (TIMEG) */
  MDX_T_OTHER,        /* zeroing, fixed-point folds, reductions */
  MDX_NTIMERS
};
int mdx_set_timers(mdx_ctx *ctx, int on);
int mdx_get_timers(mdx_ctx *ctx, double *ms, int64_t *count);

/* Measured CUDA-core FMA throughput of the current device in TFLOP/s
 * (fp64 != 0: FP64, else FP32); a roofline denominator, not a routine of the
 * reference. */
int mdx_probe_fma_peak(int fp64, double *tflops);

/* The FP64 pair sweeps' own exp(-y) and 1/d (pair_math.cuh) beside the CUDA
 * library's exp(-y) and 1.0/d, evaluated on the device for n host values
 * (y >= 0, d >= 1); a check of those routines, not a routine of the
 * reference.  Outputs: own_exp, lib_exp, own_rcp, lib_rcp (n each). */
int mdx_probe_pair_math(int n, const double *y, const double *d, double *own_exp,
                        double *lib_exp, double *own_rcp, double *lib_rcp);

#ifdef __cplusplus
}
#endif
#endif /* MDX_GPU_H */
