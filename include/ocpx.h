/*
 * ocpx.h -- C ABI of the GB300 FIM Newton-step hot path.
 *
 * Drop-in boundary for OpenCAEPoroX's fully implicit Newton step.  The
 * reference performs this work in per-cell / per-connection C++ loops driven
 * by IsoT_FIM; each entry point below replaces one of those loops over the
 * whole grid, on one GPU, with no host round trip in between:
 *
 *   ocpx_update_properties  IsoT_FIM::UpdateProperty up to the residual
 *                           (src/IsoThermalMethod.cpp:811-831): NR.CheckPhysical
 *                           ("BulkNi","BulkP"), CalFlash -> MixtureUnit::FlashFIM
 *                           per cell (src/IsoThermalMethod.cpp:1016-1071,
 *                           src/MixtureUnit.cpp:87-92), CalKrPc (:1073-1088),
 *                           CalRock (:19-30)
 *   ocpx_calres             IsoT_FIM::CalRes (src/IsoThermalMethod.cpp:1090-1185)
 *                           with OCPConvection01::CalFlux (src/OCPConvection.cpp:22-79);
 *                           the wells' terms too when they are set on the device
 *                           (PeacemanWellIsoT::CalResFIM, src/WellPeaceman.cpp:1226),
 *                           else the host adds them
 *   ocpx_assemble           IsoT_FIM::AssembleMatBulks (src/IsoThermalMethod.cpp:1187-1269)
 *                           with OCPConvection01::AssembleMatFIM (src/OCPConvection.cpp:82-187)
 *                           into LinearSystem::NewDiag/AddDiag/NewOffDiag
 *                           (include/LinearSystem.hpp:61-68), then AssembleMatWells
 *                           (:1272-1280) when the wells are on the device
 *   ocpx_newton_update      IsoT_FIM::GetSolution (src/IsoThermalMethod.cpp:1282-1418),
 *                           the wells' bhp too when they are on the device
 *   ocpx_update_last_step   IsoT_FIM::UpdateLastTimeStep, bulk part (:1473-1517)
 *   ocpx_linsolve           the linear solve of the Newton system (the wells' rows
 *                           included when they are on the device); ocpx_linsolve_async
 *                           enqueues it without waiting (capturable in a CUDA graph)
 *   ocpx_set_wells          the Peaceman wells of the deck, kept on the device
 *   ocpx_nr_*, ocpx_step_max_change, ocpx_next_time_step
 *                           Newton and time-step control (OCPNRsuite,
 *                           ControlNR, ControlTime), bulk part; see below
 *   ocpx_step               one whole Newton iteration (update, properties,
 *                           residual, Jacobian)
 *
 * Host arrays exchanged through ocpx_set_field / ocpx_get_field use the
 * reference's BulkVarSet layout (include/BulkVarSet.hpp): cell-major, then
 * phase, then component, e.g. x_ij at xij[(n*np + j)*nc + i].  The library
 * keeps its own structure-of-arrays copy in device memory.
 *
 * Errors never abort: every call returns an ocpx_status, the message of the
 * last failure in this thread is available from ocpx_last_error(), and the
 * per-cell status bits of the last property update are readable as the
 * OCPX_F_STATUS field.  One context is used by one host thread at a time.
 *
 * Wells (ocpx_set_wells) add one row and column per open well after the
 * cells, as the reference's LinearSystem orders them: the residual, the
 * Newton update and the adjoint vectors then hold nb + nwell rows of nc + 1
 * values, and the Jacobian nb + nwell block rows.
 */
#ifndef OCPX_H
#define OCPX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3: ocpx_create_ex / ocpx_options, parameters 17-19 */
#define OCPX_ABI_VERSION 3

typedef enum ocpx_status {
    OCPX_OK = 0,
    OCPX_NONCONVERGED = 1,  /* some cell's flash ended unconverged (see OCPX_F_STATUS) */
    OCPX_SINGULAR = 2,      /* a per-cell dense solve met a zero pivot */
    OCPX_NONFINITE = 3,     /* NaN/Inf in a flash result */
    OCPX_WATCHDOG = 4,      /* a device-side iteration cap was reached */
    OCPX_INVALID_ARG = 5,
    OCPX_CUDA_ERROR = 6,
    OCPX_NEGATIVE_P = 7,    /* Bulk::CheckP failed: the reference cuts the time step */
    OCPX_NEGATIVE_NI = 8,   /* Bulk::CheckNi failed: the reference cuts the time step */
    OCPX_NO_DEVICE = 9
} ocpx_status;

/* Per-cell status bits (OCPX_F_STATUS). */
#define OCPX_CELL_SPLIT_NONCONV (1u << 0)
#define OCPX_CELL_STAB_NONCONV (1u << 1)
#define OCPX_CELL_SINGULAR (1u << 2)
#define OCPX_CELL_NONFINITE (1u << 3)
#define OCPX_CELL_NEG_P (1u << 4)
#define OCPX_CELL_NEG_NI (1u << 5)
#define OCPX_CELL_ITER_CAP (1u << 6)

typedef struct ocpx_ctx ocpx_ctx;

/* A table in the reference's OCPTable storage: column-major, data[c*nrow + r]. */
typedef struct ocpx_table {
    int nrow;
    int ncol;
    const double* data;
} ocpx_table;

/* Fluid, rock and saturation model (ParamReservoir after setup). */
typedef struct ocpx_model_desc {
    int mixture;  /* 0: black-oil OGW (OCPMixtureMethodK_OGW01), 1: PR-EoS (OCPMixtureMethodComp01) */
    int nc;       /* components incl. water: 3 for black-oil, NC+1 for compositional */
    /* unit constants in force (src/OCPUnits.cpp:15-95) */
    double gravity_factor, conv_darcy, gas_constant, conv1, conv3, conv4;
    /* OCPRockIsoT_Linear */
    double rock_pref, rock_cp1, rock_cp2;
    /* SWOF (Sw, krw, krow, Pcow) and SGOF (Sg, krg, krog, Pcgo); Stone II oil */
    ocpx_table swof, sgof;
    /* PVTW (Pref, Bw, Cw, mu_w, Cmu); black-oil PVCO (Pb, Rs, Bo, mu_o, Co, Cmu), PVDG (P, Bg, mu_g) */
    ocpx_table pvtw, pvco, pvdg;
    double std_rho_o, std_rho_g, std_rho_w, std_vo, std_vg, std_vw;
    /* compositional: arrays of NC = nc-1 entries; BIC is the full NC x NC matrix;
     * Vshift already multiplied by GAS_CONSTANT*OmegaB*Tc/Pc as EoS_PR stores it */
    const double *Tc, *Pc, *Vc, *MW, *OmegaA, *OmegaB, *acf, *BIC, *Vshift, *Vcvis;
    const double* lbc_coef;   /* 5 LBC coefficients as ViscosityMethod03 stores them (x10) */
    const double* flash_ctrl; /* 13 values: SSMsta maxIt, tol, eYt, Ktol, dYtol; NRsta maxIt, tol;
                                 SSMsp maxIt, tol; NRsp maxIt, tol; RR maxIt, tol */
    int skip_psa;             /* SkipPSA enabled (reference default 1) */
} ocpx_model_desc;

/* Cells and connections (Bulk + BulkConn after Reservoir::Setup and CalTrans).
 * A subdomain of a grid split over several GPUs (BulkVarSet::nbI < nb in the
 * reference) lists its own cells first, [0, nb_interior), then its ghost
 * cells, [nb_interior, nb): copies of neighbouring subdomains' cells whose
 * properties it computes itself (the flash runs on all nb cells, as
 * IsoT_FIM::CalFlash does) but whose rows it does not own.  Residual rows,
 * residual norms, Jacobian rows and the Newton-control maxima then cover the
 * interior cells only (CalRes and AssembleMatBulks loop to nbI,
 * src/IsoThermalMethod.cpp:1095, 1197-1210; OCPNRsuite, src/OCPNRsuite.cpp:26);
 * Jacobian columns >= nb_interior are ghost columns.  Every connection needs
 * an interior end; its two ends keep their roles (bId, eId) whatever their
 * local numbers, so a subdomain's rows are bit-identical to the same rows of
 * the whole grid when its connections keep the whole grid's order. */
typedef struct ocpx_grid_desc {
    int nb;                  /* cells: interior, then ghost */
    int nconn;               /* connections, in the reference's order */
    const double* v;         /* bulk volume */
    const double* depth;
    const double* poro_init;
    const uint32_t* conn_b;
    const uint32_t* conn_e;
    const double* conn_trans; /* BulkConnPair::trans, CONV_DARCY included */
    int nb_interior;         /* cells [0, nb_interior) are interior; 0: all nb (a single domain) */
} ocpx_grid_desc;

/* State fields, reference layout.  Type: d = double, u8 = uint8 flag, u32. */
typedef enum ocpx_field {
    OCPX_F_P = 0,        /* d  [nb] */
    OCPX_F_T,            /* d  [nb]  (input temperature units) */
    OCPX_F_PB,           /* d  [nb] */
    OCPX_F_NI,           /* d  [nb*nc] */
    OCPX_F_LNI,          /* d  [nb*nc]  last time step */
    OCPX_F_NT,           /* d  [nb] */
    OCPX_F_VF,           /* d  [nb] */
    OCPX_F_VFP,          /* d  [nb] */
    OCPX_F_VFI,          /* d  [nb*nc] */
    OCPX_F_PJ,           /* d  [nb*np] */
    OCPX_F_PC,           /* d  [nb*np] */
    OCPX_F_S,            /* d  [nb*np] */
    OCPX_F_PHASE_EXIST,  /* u8 [nb*np] */
    OCPX_F_XIJ,          /* d  [nb*np*nc] */
    OCPX_F_RHO,          /* d  [nb*np] */
    OCPX_F_XI,
    OCPX_F_MU,
    OCPX_F_RHOP,
    OCPX_F_XIP,
    OCPX_F_MUP,
    OCPX_F_RHOX,         /* d  [nb*np*nc] */
    OCPX_F_XIX,
    OCPX_F_MUX,
    OCPX_F_KR,           /* d  [nb*np] */
    OCPX_F_DKRDS,        /* d  [nb*np*np] */
    OCPX_F_DPCDS,        /* d  [nb*np*np] */
    OCPX_F_DSEC_DPRI,    /* d  [nb*np*(nc+1)*(nc+1)] */
    OCPX_F_PORO,         /* d  [nb] */
    OCPX_F_POROP,
    OCPX_F_ROCKVP,
    OCPX_F_SKIP_FLAG,    /* u8 [nb] */
    OCPX_F_SKIP_MINEIG,  /* d  [nb] */
    OCPX_F_SKIP_P,
    OCPX_F_SKIP_T,
    OCPX_F_SKIP_ZI,      /* d  [nb*NC] */
    OCPX_F_STATUS,       /* u32 [nb] per-cell status bits of the last update (read only) */
    OCPX_F_FTYPE,        /* i8 [nb] flash type left by the last flash (read only) */
    OCPX_F_FLASH_ITERS,  /* i32 [nb*5] SSM-sta, NR-sta, SSM-split, NR-split, RR iterations (read only) */
    OCPX_F_UPBLOCK,      /* u32 [nconn*np] (read only) */
    OCPX_F_CONN_DP,      /* d  [nconn*np] (read only) */
    OCPX_F_FLUX_VJ,      /* d  [nconn*np] (read only) */
    OCPX_F_FLUX_NI,      /* d  [nconn*nc] (read only) */
    OCPX_F_RES,          /* d  [(nb+nwell)*(nc+1)] residual, negated as LinearSystem expects; ghost rows 0 (read only) */
    OCPX_F_RES_REL_V,    /* d  [nb] (read only) */
    OCPX_F_RES_REL_N,    /* d  [nb] (read only) */
    OCPX_F_TRANS,        /* d  [nconn] connection transmissibility (BulkConnPair::trans) */
    OCPX_F_PORO_INIT,    /* d  [nb] reference porosity (BulkVarSet::poroInit) */
    OCPX_F__COUNT
} ocpx_field;

typedef struct ocpx_report {
    uint32_t status_or;       /* OR of the per-cell status bits */
    int n_two_phase;          /* cells with two hydrocarbon phases after the flash */
    int n_flagged;            /* cells with any status bit set */
} ocpx_report;

typedef struct ocpx_norms {
    double maxRelRes_V;  /* OCPNRresidual::maxRelRes_V */
    double maxRelRes_N;
    int maxId_V;
    int maxId_N;
} ocpx_norms;

/* Context. device < 0 selects the current device. */
ocpx_status ocpx_create(const ocpx_model_desc* model, const ocpx_grid_desc* grid, int device, ocpx_ctx** out);

/* Options of ocpx_create_ex; struct_size = sizeof(ocpx_options), the other
 * fields zero for the defaults (ocpx_create's).
 *   recompute_flash_der  1: dSec_dPri (OCPMixtureMethodComp::CaldXsdXp02,
 *                        src/OCPMixtureMethodComp.cpp:565-642, np*(nc+1)^2
 *                        values per cell: 2,904 bytes at nc = 10) is not
 *                        stored.  The flash keeps the two hydrocarbon
 *                        phases' mole numbers instead (16 bytes per cell),
 *                        and the Jacobian's connection blocks, GetSolution
 *                        and the wells' perforation terms recompute it from
 *                        the state the flash left (P, T, Ni, phase labels,
 *                        x_ij) with the flash's own statements, so every
 *                        result is bit-identical to the stored form's.  The
 *                        compositional mixture only.  OCPX_F_DSEC_DPRI can
 *                        still be read (recomputed on the fly: the flash's
 *                        values until P, T or Ni change) but not written. */
typedef struct ocpx_options {
    size_t struct_size;
    int recompute_flash_der;
    int reserved[7];
} ocpx_options;
ocpx_status ocpx_create_ex(const ocpx_model_desc* model, const ocpx_grid_desc* grid, int device,
                           const ocpx_options* options, ocpx_ctx** out);
void ocpx_destroy(ocpx_ctx* ctx);
const char* ocpx_last_error(void);
int ocpx_abi_version(void);

/* Host <-> device state in the reference layout; count is the element count. */
ocpx_status ocpx_set_field(ocpx_ctx* ctx, ocpx_field f, const void* host, size_t count);
ocpx_status ocpx_get_field(ocpx_ctx* ctx, ocpx_field f, void* host, size_t count);
/* The same for the entities [first, first + n) of a field (cells, or
 * connections for the connection fields): host holds n entities in the
 * reference layout, e.g. n*np*nc values of OCPX_F_XIJ.  For reading windows of
 * a large grid and for writing a subdomain's ghost cells. */
ocpx_status ocpx_set_field_range(ocpx_ctx* ctx, ocpx_field f, size_t first, size_t n, const void* host);
ocpx_status ocpx_get_field_range(ocpx_ctx* ctx, ocpx_field f, size_t first, size_t n, void* host);

/* Newton-step pieces (asynchronous on the context stream unless noted). */
ocpx_status ocpx_update_properties(ocpx_ctx* ctx, ocpx_report* rep); /* synchronizes to fill rep */
ocpx_status ocpx_calres(ocpx_ctx* ctx, double dt, ocpx_norms* norms); /* norms may be NULL */
ocpx_status ocpx_assemble(ocpx_ctx* ctx, double dt);
ocpx_status ocpx_newton_update(ocpx_ctx* ctx, const double* u_host, double dSmax);
ocpx_status ocpx_update_last_step(ocpx_ctx* ctx);
ocpx_status ocpx_synchronize(ocpx_ctx* ctx);

/* Block-CSR Jacobian of the bulk rows in the reference's order (diagonal
 * block first, then one block per incident connection in connection order),
 * blocks (nc+1)x(nc+1) row-major. */
ocpx_status ocpx_jacobian_dims(ocpx_ctx* ctx, size_t* nrow, size_t* nnz_blocks, int* block_dim);
ocpx_status ocpx_get_jacobian(ocpx_ctx* ctx, uint32_t* rowptr, uint32_t* col, double* val);
/* Rows [r0, r1) only: rowptr receives r1 - r0 + 1 offsets into the whole
 * matrix's block arrays (rowptr[0] is the first row's), col and val the
 * blocks from rowptr[0] to rowptr[r1 - r0]; for windows of large grids. */
ocpx_status ocpx_get_jacobian_rows(ocpx_ctx* ctx, size_t r0, size_t r1, uint32_t* rowptr, uint32_t* col, double* val);
/* Device pointers of the same arrays (valid until ocpx_destroy). */
ocpx_status ocpx_jacobian_device(ocpx_ctx* ctx, const uint32_t** rowptr, const uint32_t** col, const double** val);

/* Execution variant: 0 = one kernel per reference loop (plain), 1 = batched
 * (cost-ordered flash with a work budget; over-budget cells finish their
 * phase equilibrium on whole warps).  Both give identical results. */
ocpx_status ocpx_set_variant(ocpx_ctx* ctx, int variant);

/* Tuning parameters of the execution (no effect on results):
 *   FLASH_BUDGET  work units (EoS fugacity evaluations) a cell's phase
 *                 equilibrium may use in the batched thread-per-cell flash
 *                 before it is deferred to the warp-cooperative kernel
 *                 (0 defers every cell that needs an equilibrium);
 *   COOP_BLOCKS   blocks of the warp-cooperative kernel;
 *   BLOCK_CELL    threads per block of the per-cell kernels;
 *   DEFERRED      (read only) cells whose equilibrium ran on the
 *                 warp-cooperative kernel in the last batched flash
 *                 (pre-deferred, and left over after the rounds);
 *                 reading it synchronizes the context stream;
 *   PREDEFER      cells whose last flash used more than this many work
 *                 units go to the cooperative kernel at once, on a second
 *                 stream, while the per-cell kernel runs (default 192);
 *                 0: only cells that exceed the budget now are deferred;
 *   COOP_CELLS    adaptive floor of both thresholds, active only when
 *                 more than this many cells are predicted above the
 *                 pre-deferral threshold (the budget when PREDEFER is 0):
 *                 then about this many of the cells with the largest
 *                 predicted work go to the cooperative kernel and the
 *                 per-cell kernel keeps the rest (default 1216, two per warp
 *                 slot).  0: the thresholds are the two parameters above
 *                 only;
 *   PREDEFERRED   (read only) cells of DEFERRED that were pre-deferred;
 *   LEVEL         (read only) the adaptive work level of the last batched
 *                 flash (0: no floor; else the budget was at least
 *                 2^(LEVEL/4) work units);
 *   PRE_BLOCKS    > 0: the pre-deferred cells run on this many SM-exclusive
 *                 blocks (one warp per SM sub-partition, no other block on
 *                 the SM while they run) instead of COOP_BLOCKS blocks that
 *                 share SMs with the per-cell kernel (default 0);
 *   CELL_BLOCKS   > 0: the budgeted per-cell kernel runs as this many
 *                 persistent blocks whose warps take 32 cells at a time in
 *                 cost order (fewer resident warps, dynamic balance);
 *                 0: one thread per cell (default);
 *   ROUNDS        re-budgeting rounds (0..8, default 0): the cells over the
 *                 budget are rerun one thread per cell, compacted, with the
 *                 budget multiplied by ROUND_GROWTH per round, before the
 *                 cells left over go to the cooperative kernel; with rounds
 *                 the adaptive floor no longer raises the budget (it still
 *                 limits pre-deferral);
 *   ROUND_GROWTH  budget factor per round (2..64, default 4);
 *   FUSED_BLOCKS  > 0: the batched flash as one persistent kernel of this
 *                 many blocks of four warps (one block per SM holds the SM
 *                 alone when the count is at most the SM count).  Its warps
 *                 run the pre-deferred cells cooperatively, then the
 *                 cost-ordered cells one per lane with the budget, then the
 *                 over-budget cells cooperatively as they are published;
 *                 no second stream (default: the SM count below 131,072
 *                 cells, four times it from there on).  0: the
 *                 two-stream form (PRE_BLOCKS, CELL_BLOCKS, ROUNDS and
 *                 COOP_BLOCKS apply to it only);
 *   SMS           (read only) SMs of the context's device;
 *   FUSED_COOP_BLOCKS  > 0: the first this many fused blocks run only the
 *                 cooperative work (pre-deferred cells, then over-budget
 *                 cells as they are published, waiting for them within a
 *                 bound), the others the per-lane cells, so the long chains
 *                 never share an SM with per-lane work.  The launch is then
 *                 cooperative: FUSED_BLOCKS must be at most the SM count (one
 *                 block per SM, all resident at once) and larger than this
 *                 value.  -1 (default): half of FUSED_BLOCKS below
 *                 131,072 cells when FUSED_BLOCKS is at most the SM count,
 *                 else 0; reading the parameter gives the value in effect;
 *   FUSED_EXCL    1: fused blocks that number at most the SM count reserve
 *                 all of an SM's shared memory, so each holds an SM alone;
 *                 0 (default): no reservation, and the SMs keep the largest
 *                 L1 cache the static shared memory allows, where the
 *                 per-lane cells' thread frames live (36,000 cells: fused
 *                 kernel 10.4 ms against 11.2 ms);
 *   POST_BLOCK    threads per block of the kernel that finishes the deferred
 *                 cells from their equilibrium (32, 64, 96 or 128; default
 *                 32: one warp per SM keeps its frames in L1);
 *   RECOMPUTE_FLASH_DER  (read only) 1 when the context was created with
 *                 ocpx_options.recompute_flash_der;
 *   DEVICE_BYTES  (read only) device memory the context holds: its arena,
 *                 the linear system, the wells, the solver's and the
 *                 adjoint's work space and the checkpoints;
 *   SPLIT_REFILL  1: in the fused form, the cells whose flash starts with
 *                 the phase split run the split's first successive-
 *                 substitution loop in a kernel whose lanes take a new cell
 *                 as soon as theirs is done, then the rest of their flash
 *                 from the saved state; results bit-identical.  Allocates
 *                 one saved state per cell (704 bytes) when first set.
 *                 0 (default): off. */
typedef enum ocpx_param {
    OCPX_PARAM_FLASH_BUDGET = 0,
    OCPX_PARAM_COOP_BLOCKS = 1,
    OCPX_PARAM_BLOCK_CELL = 2,
    OCPX_PARAM_DEFERRED = 3,
    OCPX_PARAM_PREDEFER = 4,
    OCPX_PARAM_COOP_CELLS = 5,
    OCPX_PARAM_PREDEFERRED = 6,
    OCPX_PARAM_LEVEL = 7,
    OCPX_PARAM_PRE_BLOCKS = 8,
    OCPX_PARAM_CELL_BLOCKS = 9,
    OCPX_PARAM_ROUNDS = 10,
    OCPX_PARAM_ROUND_GROWTH = 11,
    OCPX_PARAM_FUSED_BLOCKS = 12,
    OCPX_PARAM_SMS = 13,
    OCPX_PARAM_FUSED_COOP_BLOCKS = 14,
    OCPX_PARAM_FUSED_EXCL = 15,
    OCPX_PARAM_POST_BLOCK = 16,
    OCPX_PARAM_RECOMPUTE_FLASH_DER = 17,
    OCPX_PARAM_DEVICE_BYTES = 18,
    OCPX_PARAM_SPLIT_REFILL = 19
} ocpx_param;
ocpx_status ocpx_set_param(ocpx_ctx* ctx, ocpx_param p, long long value);
ocpx_status ocpx_get_param(ocpx_ctx* ctx, ocpx_param p, long long* value);

/* One Newton iteration: optional host Newton update u ((nb+nwell)*(nc+1), may be
 * NULL), then properties, residual and Jacobian; optional host copies of the
 * residual ((nb+nwell)*(nc+1)) and Jacobian block values.  Synchronizes. */
ocpx_status ocpx_step(ocpx_ctx* ctx, const double* u_host, double dSmax, double dt, double* res_host,
                      double* jac_val_host, ocpx_report* rep);

/* Asynchronous form of ocpx_step without host buffers: enqueue properties,
 * residual and Jacobian on the context stream and return at once;
 * ocpx_step_report then waits and reads the status summary.  In the batched
 * variant the sequence is captured into a CUDA graph on first use (again
 * after dt, the variant or a tuning parameter changes) and replayed with one
 * launch; while stage profiling is on it runs kernel by kernel. */
ocpx_status ocpx_enqueue_step(ocpx_ctx* ctx, double dt);
ocpx_status ocpx_step_report(ocpx_ctx* ctx, ocpx_report* rep);

/* Per-stage device timing with CUDA events recorded on the context stream.
 * Stages: 0 physical check, 1 flash, 2 kr/Pc + rock, 3 status summary,
 * 4 connection flux, 5 residual + norms, 6 Jacobian connection blocks,
 * 7 Jacobian rows, 8 Newton update; inside stage 1 of the batched form:
 * 9 pre-deferral and cost order, 10 budgeted per-cell flash, 11 cooperative
 * equilibrium and properties of the pre-deferred cells (second stream,
 * concurrent with 10), 12 properties of the cells deferred by 10,
 * 13 cooperative equilibrium of the cells deferred by 10; 14 the adjoint
 * products of the step (ocpx_set_adjoint_seed).  ocpx_profile_read synchronizes and returns, per
 * stage, the summed milliseconds and the number of timed launches since
 * profiling was enabled. */
#define OCPX_STAGE_COUNT 15
ocpx_status ocpx_profile_enable(ocpx_ctx* ctx, int enable);
ocpx_status ocpx_profile_read(ocpx_ctx* ctx, double* ms, uint64_t* launches);

/* Save (restore = 0) or restore (restore = 1) the whole mutable bulk state
 * (every per-cell array) in device-side slot 0 or 1.  Restoring slot 0 after
 * saving it at the start of a time step is IsoT_FIM::ResetToLastTimeStep
 * (src/IsoThermalMethod.cpp:1420-1471) without any host copy. */
ocpx_status ocpx_checkpoint(ocpx_ctx* ctx, int slot, int restore);

/* Measured FP64 fused multiply-add throughput of the device (TFLOP/s), the
 * roofline denominator of the FP64-bound flash; iters sets the run length. */
ocpx_status ocpx_measure_fp64_tflops(int device, int iters, double* tflops);

/* Relative-residual norms with no allocation at all.  No counterpart in the
 * reference: it is the "Calculate RelRes" loop of IsoT_FIM::CalRes
 * (src/IsoThermalMethod.cpp:1147-1167) as a context-free call on device
 * arrays, for callers that hold a residual on the device but cannot allocate
 * device memory at that point (their allocator owns the device, or the
 * implicit device-wide synchronisation of cudaMalloc/cudaFree would stall
 * their other streams).
 *   d_res [nb*len] residual (either sign), d_rockVp [nb], d_Nt [nb]: inputs;
 *   d_resRelV, d_resRelN [nb]: outputs (per-cell norms, as ocpx_calres);
 *   norms (host): maxRelRes_V/N and maxId_V/N, first cell wins ties.
 * Runs on `stream` (a cudaStream_t, NULL = default stream) and waits for it.
 * Its reduction scratch is one static device array per process and device
 * (OCPX_RELRES_NOALLOC_MAX_BLOCKS partials, about 24 KB); nb above
 * OCPX_RELRES_NOALLOC_MAX_CELLS returns OCPX_INVALID_ARG.  The scratch's
 * block counter starts at zero and every call leaves it at zero.  Calls
 * whose kernels overlap in time race on the scratch: serialise them (one
 * stream).  Every call looks up the scratch's address in the current
 * device's context (cudaGetSymbolAddress, which allocates nothing); the first
 * call on a device may load the library's module there, so make it outside
 * any stream capture.  Errors are
 * returned as status only; ocpx_last_error is not updated. */
#define OCPX_RELRES_NOALLOC_MAX_BLOCKS 1024
#define OCPX_RELRES_NOALLOC_MAX_CELLS 2097152
ocpx_status ocpx_relres_noalloc(const double* d_res, const double* d_rockVp, const double* d_Nt, int nb, int len,
                                double* d_resRelV, double* d_resRelN, void* stream, ocpx_norms* norms);

/* Adjoint of the bulk residual R (the negated residual of ocpx_calres) at the
 * state of the last ocpx_assemble, as vector-Jacobian products with a host
 * vector lambda [(nb+nwell)*(nc+1)] (cell-major, like the residual).  No counterpart
 * in the reference, which has no adjoint:
 *   jt_lambda  [(nb+nwell)*(nc+1)]  J^T lambda, J the assembled Jacobian dR/d(P, Ni);
 *   dr_dtrans  [nconn]      (dR/dT_c)^T lambda for every connection's
 *                           transmissibility (R is linear in T_c: the flux of
 *                           OCPConvection01::CalFlux scales with it);
 *   dr_dporo   [nb]         (dR/dporoInit_n)^T lambda (only the volume balance
 *                           depends on it, through OCPRockIsoT_Linear::CalPoro).
 * Outputs may be NULL.  Synchronizes. */
ocpx_status ocpx_adjoint(ocpx_ctx* ctx, const double* lambda, double* jt_lambda, double* dr_dtrans,
                         double* dr_dporo);
/* The same products as part of every Newton step: with a seed set, each
 * ocpx_enqueue_step / ocpx_step computes J^T lambda, (dR/dT)^T lambda and
 * (dR/dporoInit)^T lambda on the device right after its Jacobian (inside the
 * step's graph in the batched variant), and ocpx_get_adjoint copies the last
 * step's products to the host (any pointer may be NULL; synchronizes).  The
 * seed [(nb+nwell)*(nc+1)] is copied to the device once; NULL turns the products off.
 * The first seed allocates their device buffers (2*(nb+nwell)*(nc+1) + nb + nconn
 * doubles).  ocpx_adjoint keeps its own buffers and leaves the seed alone. */
ocpx_status ocpx_set_adjoint_seed(ocpx_ctx* ctx, const double* lambda);
ocpx_status ocpx_get_adjoint(ocpx_ctx* ctx, double* jt_lambda, double* dr_dtrans, double* dr_dporo);

/* Newton-iteration and time-step control of the FIM run, bulk part, on the
 * device.  Replaces, for the bulk cells:
 *   ocpx_nr_init_step       OCPNRsuite::InitStep (src/OCPNRsuite.cpp:70-83):
 *                           the last Newton iterate := the last time step's
 *                           state (saved by ocpx_update_last_step), and the
 *                           initial residual norm := that of the last
 *                           ocpx_calres (CalInitRes, src/IsoThermalMethod.cpp:1170-1177)
 *   ocpx_nr_max_change      OCPNRsuite::CalMaxChangeNR (src/OCPNRsuite.cpp:86-160)
 *   ocpx_step_max_change    OCPNRsuite::CalMaxChangeTime (src/OCPNRsuite.cpp:163-232)
 *   ocpx_nr_check_converge  ControlNR::CheckConverge with {"res", "d"}
 *                           (src/OCPControlNR.cpp:27-77), as IsoT_FIM::FinishNR
 *                           calls it (src/IsoThermalMethod.cpp:838-864)
 *   ocpx_next_time_step     ControlTime::CalNextTimeStep with {"dP", "dS", "iter"}
 *   ocpx_wells_eval         PeacemanWell(IsoT) CalTrans, CalFlux, CalResFIM,
 *                           AssembleMatInjFIM / AssembleMatProdFIM
 *                           (src/OCPControlTime.cpp:128-178), as IsoT_FIM::FinishStep
 *                           calls it (src/IsoThermalMethod.cpp:865-870)
 * The maxima are signed, with the reference's rule: the first entry in cell
 * order whose magnitude is the largest, 0 when every change is 0; results
 * are bit-identical to the reference's.  Without ocpx_set_wells the wells
 * stay with the host, and their terms enter through ocpx_nr_control; with
 * it, ocpx_nr_check_converge uses the device's maxWellRelRes_mol (unless
 * res_from_host).  Every output pointer may be NULL: the values then stay
 * on the device for the next call, and nothing synchronizes. */
typedef struct ocpx_change_max {
    double dP, dT, dN, dS, eV;  /* pressure, temperature, relative moles, saturation, volume error */
} ocpx_change_max;
typedef struct ocpx_nr_control {
    /* ControlNRParam (include/OCPControlNR.hpp:28-51) */
    int maxIter;
    double tol, dPmin, dSmin;
    /* ControlTimeParam (include/OCPControlTime.hpp:29-72) */
    double maxIncreFac, minChopFac, dPlim, dSlim, timeMax, timeMin, end_time;
    /* the time step that ends: its length and the time at its start */
    double current_dt, current_time;
    /* Newton iterations done in this time step (OCPNRsuite::GetIterNR) */
    int iterNR;
    /* well terms: the largest relative well-equation residual
     * (OCPNRresidual::maxWellRelRes_mol) and the well pressure change over the
     * time step that CalMaxChangeTime compares with the bulk's (dPWmaxT) */
    double maxWellRelRes_mol, dPWmaxT;
    /* 1: use these residual norms (for example with the wells' perforation
     * terms added by the host); 0: the device's, from the last ocpx_calres
     * and the one recorded by ocpx_nr_init_step */
    int res_from_host;
    double maxRelRes_V, maxRelRes0_V, maxRelRes_N;
} ocpx_nr_control;
ocpx_status ocpx_nr_init_step(ocpx_ctx* ctx);
ocpx_status ocpx_nr_max_change(ocpx_ctx* ctx, ocpx_change_max* out);
ocpx_status ocpx_step_max_change(ocpx_ctx* ctx, ocpx_change_max* out);
/* state: 0 converged, 1 keep iterating, 2 not converged within maxIter
 * (the integer values of the reference's OCPNRStateC) */
ocpx_status ocpx_nr_check_converge(ocpx_ctx* ctx, const ocpx_nr_control* c, int* state);
/* next_dt: the length of the next time step (clamped to the end of the
 * current report interval, end_time); predict_dt: the same before that clamp */
ocpx_status ocpx_next_time_step(ocpx_ctx* ctx, const ocpx_nr_control* c, double* next_dt, double* predict_dt);

/* Peaceman wells: the wells' part of the residual and of the Jacobian,
 * computed on the device from the context's current bulk state (kr, mu, xi,
 * xij and their derivatives, dSec_dPri) and, for the residual, its last
 * ocpx_calres.  Replaces PeacemanWell::CalTrans / CalFlux and
 * PeacemanWellIsoT::CalResFIM / AssembleMatInjFIM / AssembleMatProdFIM
 * (src/WellPeaceman.cpp:365-466, 1226-1361, 1488-1613) for open wells; the
 * unweighted-permeability option is not supported.  Inputs the reference
 * computes at well setup or from the mixture are passed in: WI*multiplier and
 * dG per perforation, the injected fluid's molar density per perforation, the
 * rate-control factors (CalFactor). */
typedef struct ocpx_well {
    int type;               /* 0 injector, 1 producer */
    int mode;               /* 0 BHP control, 1 rate control */
    double bhp, tar_bhp, tar_rate;
    int nperf;
    const int* cell;        /* [nperf] perforated cells */
    const double* WI;       /* [nperf] WI * multiplier */
    const double* dG;       /* [nperf] perforation pressure minus bhp */
    const double* xi_inj;   /* [nperf] injected fluid molar density (injectors) */
    const double* inj_zi;   /* [nc] injected composition (injectors) */
    const double* factor;   /* [nc] rate factors (rate control) */
} ocpx_well;
/* res_out [(nb + nwell) * (nc + 1)], may be NULL: the residual with the
 * wells, in the reference's sign (IsoT_FIM::CalRes negates it), well w's row
 * at nb + w.  blocks_out, may be NULL: (nc + 1)^2 values, row-major, per
 * block: for each perforation in order the block added to its cell's
 * diagonal, the cell-to-well block (row cell, column nb + w) and the
 * well-to-cell block (row nb + w, column cell); then each well's diagonal
 * block.  max_rel, may be NULL: maxWellRelRes_mol.  res_out needs an
 * ocpx_calres at the current state (after the last property update, field
 * write, Newton update or checkpoint restore): otherwise OCPX_INVALID_ARG.
 * For a host that keeps its own well code; see ocpx_set_wells for the wells
 * inside the step. */
ocpx_status ocpx_wells_eval(ocpx_ctx* ctx, int nwell, const ocpx_well* wells, double dt, double* res_out,
                            double* blocks_out, double* max_rel);

/* Peaceman wells inside the Newton step.  The well set (types, controls,
 * targets, perforations with WI*multiplier and dG, injected fluid, rate
 * factors, and each well's current bhp) is copied to the device; from then on
 * ocpx_calres, ocpx_assemble, ocpx_step and the step's graph add the wells'
 * terms on the device after the bulk rows, in the reference's order
 * (IsoT_FIM::CalRes with PeacemanWellIsoT::CalResFIM, src/WellPeaceman.cpp:
 * 1226-1265; IsoT_FIM::AssembleMatWells, src/IsoThermalMethod.cpp:1272-1280,
 * with AssembleMatInjFIM / AssembleMatProdFIM, src/WellPeaceman.cpp:1268-1361,
 * 1488-1613): each perforated cell's residual rows and diagonal block, one
 * bulk-to-well block per perforation after the cell's connection blocks, and
 * per open well w a row nb + w (its control equation; diagonal block, then one
 * well-to-bulk block per perforation).  ocpx_assemble uses the perforation
 * terms of the last ocpx_calres, as the reference assembles from the state
 * its residual was computed at.  The Newton update adds u of row nb + w to
 * well w's bhp (GetSolutionFIM, :1198-1204); the checkpoints carry the bhp;
 * the device linear solve and the adjoint cover the wells' rows.  Call it
 * again when a control switches or a new time step changes dG: with the same
 * perforations nothing is reallocated, otherwise the system's storage is
 * rebuilt (its contents and any adjoint seed are dropped).  nwell = 0 removes
 * the wells.  Single domain only (no ghost cells); ocpx_wells_eval is refused
 * while wells are set.  ocpx_get_wells reads each well's bhp and the
 * maxWellRelRes_mol of the last ocpx_calres (synchronizes).  The
 * unweighted-permeability option is not supported. */
ocpx_status ocpx_set_wells(ocpx_ctx* ctx, int nwell, const ocpx_well* wells);
ocpx_status ocpx_get_wells(ocpx_ctx* ctx, double* bhp, double* max_rel);

/* Linear solve of the Newton system on the device: J u = rhs, J the bulk
 * Jacobian of the last ocpx_assemble and rhs the residual of the last
 * ocpx_calres as the reference passes it to its solver (LinearSystem::CopyRhs
 * of the negated residual, src/IsoThermalMethod.cpp:742-752).  The reference
 * hands this system to an external package (FASP, PETSc or PARDISO,
 * src/LinearSystem.cpp:35-89); here BiCGStab with right block-Jacobi
 * preconditioning, from u = 0, until |rhs - J u| <= tol |rhs| or maxit
 * iterations (the norm is tested on the device every 10).  The system holds the wells'
 * rows when ocpx_set_wells gave them; a host that keeps its own well code
 * solves the full system itself.  Single domain only.  The solution stays on
 * the device for ocpx_newton_update_device and is copied to u_host
 * ((nb+nwell)*(nc+1)) when that is not NULL.  The first call allocates the solver's work space
 * (about 8 vectors and the inverted diagonal blocks).  Synchronizes. */
typedef struct ocpx_solve_report {
    int iterations;
    double relres;   /* of the recursively updated residual */
    int converged;
    int breakdown;   /* 1: BiCGStab breakdown, 2: a singular diagonal block */
} ocpx_solve_report;
ocpx_status ocpx_linsolve(ocpx_ctx* ctx, double tol, int maxit, double* u_host, ocpx_solve_report* rep);
/* The same solve, enqueued on the context stream without waiting: the
 * convergence test runs on the device every 10 iterations and, once the
 * solve has converged or broken down, the rest of the maxit iterations'
 * kernels return at once.  No host synchronization, allocation or host
 * memory access once the work space exists (the first solve of either form
 * allocates it and must not run inside a stream capture), so the call can be
 * captured in a CUDA graph on the context stream (ocpx_stream).  The solution
 * and the report are the same as ocpx_linsolve's. */
ocpx_status ocpx_linsolve_async(ocpx_ctx* ctx, double tol, int maxit);
/* Waits for the context stream and reads the report of the last solve. */
ocpx_status ocpx_linsolve_report(ocpx_ctx* ctx, ocpx_solve_report* rep);
/* IsoT_FIM::GetSolution, bulk part, with the update the last ocpx_linsolve
 * left on the device. */
ocpx_status ocpx_newton_update_device(ocpx_ctx* ctx, double dSmax);

/* Stream the context launches on (a cudaStream_t), for callers that time or
 * order work around the library. */
void* ocpx_stream(ocpx_ctx* ctx);
/* Number of kernels the library launched on this context so far. */
uint64_t ocpx_launch_count(ocpx_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* OCPX_H */
