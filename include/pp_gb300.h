/*
 * pp_gb300.h -- C ABI of the GB300-native bond-based peridynamics time step.
 *
 * Every entry point takes device pointers (allocated by the caller), sizes,
 * scalars and a CUDA stream passed as `void*` (NULL = the legacy default
 * stream).  Nothing here allocates device memory, synchronises the stream or
 * throws; each call returns PP_SUCCESS or one of the PP_ERROR_* codes below,
 * and pp_status_string() turns a code into text.  Launch errors are read
 * with cudaGetLastError() right after the launch and returned as
 * PP_ERROR_CUDA; asynchronous kernel faults surface at the caller's next
 * synchronisation, as for any CUDA library.
 *
 * Array layouts follow PeriPy's device integrators (peripy/integrators.py
 * :84-254): node arrays are row-major (nnodes, 3) float64 or int32, the
 * neighbour list is (nnodes, max_neigh) int32 padded and broken with -1,
 * max_neigh a power of two (peripy/model.py:575-578).
 *
 * Each declaration names the reference interface it replaces.
 */
#ifndef PP_GB300_H
#define PP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PP_ABI_VERSION 3

/* Status codes. */
#define PP_SUCCESS                  0
#define PP_ERROR_INVALID_VALUE      1  /* bad size, NULL pointer or flag   */
#define PP_ERROR_MAX_NEIGH          2  /* max_neigh not a power of 2 <= 1024 */
#define PP_ERROR_MISALIGNED         3  /* pointer not aligned as required  */
#define PP_ERROR_UNSUPPORTED        4  /* option combination not built     */
#define PP_ERROR_CUDA               5  /* a CUDA runtime call failed       */
#define PP_ERROR_TOO_LARGE          6  /* more steps than the static scratch holds */

/* Integrator kinds (peripy/integrators.py:462, 544, 651). */
#define PP_EULER                    0
#define PP_EULER_CROMER             1
#define PP_VELOCITY_VERLET          2

/* Arithmetic of the fused step. */
#define PP_FLOAT64                  0  /* IEEE binary64 throughout          */
#define PP_MIXED                    1  /* FP32 bonds, exact FP64 stretch test,
                                          double-float node state          */

/* Number of PP_MIXED kernel variants (pp_fused_args.variant). */
#define PP_MIXED_VARIANTS           3

/* Values of pp_fused_args.status after a step (read by the caller).  The
 * word reports errors that a kernel detects on the device; a kernel with a
 * bounded wait sets PP_STATUS_COPY_TIMEOUT when the wait runs out.  The
 * PP_MIXED step of this version has no waits and leaves PP_STATUS_OK.     */
#define PP_STATUS_OK                0
#define PP_STATUS_COPY_TIMEOUT      1  /* a wait for an asynchronous copy ran
                                          out: the step's results are invalid */
#define PP_STATUS_BAD_TILING        2  /* a tile exceeded PP_TILE_NODES_MAX or
                                          its halo capacity: it was skipped,
                                          the step's results are invalid   */

/* Flags of the fused step. */
#define PP_FLAG_COMPENSATED         1  /* PP_MIXED only: compensated FP32 force
                                          sums (FMA product error + TwoSum,
                                          carried through the warp reduction);
                                          PP_ERROR_UNSUPPORTED with PP_FLOAT64 */

/* ------------------------------------------------------------------------ */
/* Utility.                                                                 */
/* ------------------------------------------------------------------------ */

/* Text for a status code (static storage). */
const char* pp_status_string(int status);

/* PP_ABI_VERSION of the loaded library. */
int pp_abi_version(void);

/* ------------------------------------------------------------------------ */
/* Reference-structured FP64 kernels ("plain" step).                        */
/* Same arithmetic, in the same operation order and with the same           */
/* work-group tree reduction order, as PeriPy's OpenCL kernels; separate    */
/* launches for bond force, displacement update and damage.                 */
/* ------------------------------------------------------------------------ */

typedef struct pp_bond_force_args {
    int32_t nnodes;
    int32_t max_neigh;             /* power of two, 1..1024               */
    int32_t nregimes;              /* used when bond_types != NULL         */
    int32_t nbond_types;           /* used when bond_types != NULL         */
    const double* u;               /* (nnodes,3)                           */
    double* force;                 /* (nnodes,3) out                       */
    double* body_force;            /* (nnodes,3) out                       */
    const double* r0;              /* (nnodes,3)                           */
    const double* vols;            /* (nnodes)                             */
    int32_t* nlist;                /* (nnodes,max_neigh) in/out, -1 broken */
    const int32_t* fc_types;       /* (nnodes,3)                           */
    const double* fc_values;       /* (nnodes,3)                           */
    const double* stiffness_corrections; /* (nnodes,max_neigh) or NULL     */
    const int32_t* bond_types;     /* (nnodes,max_neigh) or NULL           */
    int32_t* regimes;              /* (nnodes,max_neigh) in/out; with bond_types */
    const double* plus_cs;         /* (nbond_types*nregimes); with bond_types */
    const double* bond_stiffness_table;   /* (nbond_types*nregimes); with bond_types */
    const double* critical_stretch_table; /* (nbond_types*nregimes); with bond_types */
    double bond_stiffness;         /* scalar; without bond_types           */
    double critical_stretch;       /* scalar; without bond_types           */
    double fc_scale;               /* force_bc_magnitude of this step      */
} pp_bond_force_args;

/* Replaces bond_force1..bond_force4 (peripy/cl/peridynamics.cl:4-565),
 * selected as peripy/integrators.py:109-148 does: by whether
 * stiffness_corrections and bond_types are NULL. */
int pp_bond_force(const pp_bond_force_args* args, void* stream);

/* Replaces damage (peripy/cl/peridynamics.cl:568-610):
 * n_neigh[i] = intact slots of row i, damage[i] = 1 - n_neigh[i]/family[i]. */
int pp_damage(const int32_t* nlist, const int32_t* family, int32_t* n_neigh,
              double* damage, int32_t nnodes, int32_t max_neigh,
              void* stream);

/* Replaces update_displacement of peripy/cl/euler.cl:3-24 (one DOF per
 * element, ndof = 3*nnodes). */
int pp_update_displacement_euler(const double* force, double* u,
                                 const int32_t* bc_types,
                                 const double* bc_values, double bc_scale,
                                 double dt, int64_t ndof, void* stream);

/* Replaces update_displacement of peripy/cl/euler_cromer.cl:3-35. */
int pp_update_displacement_euler_cromer(
    const double* force, double* u, double* ud, double* udd,
    const int32_t* bc_types, const double* bc_values,
    const double* densities, double bc_scale, double damping, double dt,
    int64_t ndof, void* stream);

/* Replaces update_displacement of peripy/cl/velocity_verlet.cl:3-36. */
int pp_update_displacement_velocity_verlet(
    const double* force, double* u, double* ud, double* udd,
    const int32_t* bc_types, const double* bc_values,
    const double* densities, double bc_scale, double damping, double dt,
    int64_t ndof, void* stream);

/* ------------------------------------------------------------------------ */
/* Fused step: one launch per time step does stretch, break (n-linear       */
/* regimes), force, per-node reduction, force boundary conditions, intact   */
/* count and the integrator update.  Replaces the launch pair of            */
/* EulerCL/EulerCromerCL/VelocityVerletCL.__call__                          */
/* (peripy/integrators.py:484-503, 586-606, 700-720).                       */
/*                                                                          */
/* Displacements are double-buffered: a step reads state slot `parity` and  */
/* writes slot `parity ^ 1`, so no node reads a displacement another node   */
/* has already advanced.                                                    */
/*                                                                          */
/* PP_FLOAT64 keeps the reference layouts: u[2] (nnodes,3) f64, ud, udd,    */
/* force, body_force (nnodes,3) f64, n_neigh and damage per node.  Bond     */
/* arithmetic is bit-identical to the plain kernels.                        */
/*                                                                          */
/* PP_MIXED uses the compact layouts produced by pp_mixed_pack():           */
/*   rec[2]  (nnodes) 32-byte node records, 32-byte aligned, gathered by    */
/*           the neighbours of a node with one 256-bit load:               */
/*           {qx,qy,qz (int32), w, ux,uy,uz, m (float)}.  q: fixed-point    */
/*           positions, r0 = origin + q * pos_scale, pos_scale a power of   */
/*           two with pos_scale >= 2^-21 * pp_bond_extent() so that every   */
/*           bond's |q[j] - q[i]| < 2^22 converts to float exactly without  */
/*           an int-to-float instruction; w = k*vol (PMB) or vol (bond      */
/*           types); u = FP32 displacement (high part of the double-float   */
/*           pair); m = max|u| of the node.  The step reads rec[parity] and */
/*           writes the whole of rec[parity ^ 1].                           */
/*   ulo[2]  (nnodes) float4: low parts of the double-float displacement    */
/*   vel     (nnodes) float4 x2 {hi; lo}: double-float velocity (EC, VV)    */
/*   acc     (nnodes) float4: FP32 acceleration (EC, VV)                    */
/*   frc     (nnodes) float4 x2 {force; body_force} FP32                    */
/*   rho32   (nnodes) float4 FP32 reciprocal densities 1/rho (EC, VV)       */
/*   nflags  (nnodes) int: bit d set when bc_types[3i+d] != 0, bit 3+d when  */
/*           fc_types[3i+d] != 0                                            */
/*   sc32    (nnodes,max_neigh) float stiffness corrections or NULL         */
/* umax and status are caller-allocated device words (zero-initialised by   */
/* pp_mixed_pack / the caller) that the step reads and updates.             */
/* The step reads the reference r0 (f64) and the double-float displacement  */
/* only                                                                     */
/* for bonds whose FP32 stretch lies within a proven error band of a        */
/* critical stretch; there the break/regime decision is taken from the      */
/* binary64 stretch formula of peridynamics.cl:65-75, so it is the          */
/* decision binary64 arithmetic makes on the same state.                    */
/* pp_mixed_export() writes the reference-layout f64 arrays.                */
/* ------------------------------------------------------------------------ */

/* ------------------------------------------------------------------------ */
/* Tiled layout of the PP_MIXED step (no counterpart in the reference,      */
/* whose kernels gather every neighbour from global memory).                */
/*                                                                          */
/* The nodes are renumbered internally ("internal order": internal node i  */
/* is reference node perm[i]) and cut into tiles, ranges [tile_start[t],    */
/* tile_start[t+1]) of at most PP_TILE_NODES_MAX internal nodes.  The halo  */
/* of a tile is the ascending list of internal nodes its bonds reach (its   */
/* own nodes included), at most halo_cap long.  A step stages each tile's   */
/* halo records in shared memory once and gathers every bond of the tile   */
/* from there.  Row i holds the bonds of internal node i as 16-bit entries, */
/* each 16 x the halo index of the neighbour (the byte offset of its staged */
/* record); a broken bond or padding holds the entry of node i itself.     */
/* Rows follow the reference row's slot order, CSR-packed: row i occupies   */
/* [16 row_off[i], 16 row_off[i+1]), its length the number of its intact   */
/* slots rounded up to 16.  Row entry p = 16 m + 8 h + l (l < 8, h < 2) is  */
/* stored at position 16 m + 2 l + h of the row, so that lane l of a node's */
/* eight lanes reads its entries 16 m + l and 16 m + 8 + l with one 32-bit  */
/* load.  Any permutation and any cut into ranges gives the same results;   */
/* spatial locality of the tiles only makes the step faster.  (A node      */
/* listed as its own neighbour is held as a broken bond from the start;    */
/* the reference breaks it in the first step, its stretch being 0/0.)      */
/*                                                                          */
/* The caller allocates every array and chooses perm and tile_start;       */
/* pp_tile_halos and pp_tile_rows fill the rest from the reference layouts. */
/* The step trusts the entries as it trusts a reference neighbour list:    */
/* they must be those pp_tile_rows wrote, as the steps since have left them. */
/* ------------------------------------------------------------------------ */

#define PP_TILE_NODES_MAX           128   /* internal nodes per tile       */
#define PP_TILE_HALO_MAX            768   /* largest halo_cap: 32 bytes of
                                             shared memory per record      */

typedef struct pp_tiling {
    int32_t ntiles;
    int32_t halo_cap;          /* halo capacity per tile, 1..PP_TILE_HALO_MAX */
    const int32_t* perm;       /* (nnodes) internal -> reference node      */
    const int32_t* inv;        /* (nnodes) reference -> internal node      */
    const int32_t* tile_start; /* (ntiles + 1), tile_start[0] = 0,
                                  tile_start[ntiles] = nnodes             */
    int32_t* halo;             /* (ntiles * halo_cap) internal nodes       */
    int32_t* halo_count;       /* (ntiles) halo lengths (pp_tile_halos)    */
    int32_t* own_off;          /* (ntiles) halo index of the tile's first node */
    int32_t* tile_ref;         /* (ntiles * 4) the tile's reference point in
                                  fixed-point steps (x, y, z, 0): staged
                                  positions are float(q - ref) * pos_scale,
                                  exact because |q - ref| < 2^22          */
    int32_t* row_off;          /* (nnodes + 1) row offsets, units of 16 entries */
    uint16_t* entry;           /* (16 row_off[nnodes]) 16 x halo index     */
    uint8_t* slot;             /* same length: the entry's slot in the
                                  reference row, 0xFF for padding         */
    uint8_t* bond_type;        /* same length, or NULL without bond types  */
    uint8_t* regime;           /* same length, or NULL without bond types  */
    float* correction;         /* same length, or NULL without stiffness
                                  corrections (rounded to float)          */
    double* r0;                /* (nnodes, 3) internal order               */
    double* bc_values;         /* (nnodes, 3) internal order               */
    double* fc_values;         /* (nnodes, 3) internal order               */
    int32_t* node_instance;    /* (nnodes) internal order, or NULL         */
    int32_t* n_neigh;          /* (nnodes) internal order: intact bonds
                                  after a step                            */
    int32_t* sched;            /* two device words, zero before the first
                                  step (pp_tile_rows zeroes them); the step
                                  hands out tiles with them and leaves them
                                  zero                                    */
} pp_tiling;

typedef struct pp_fused_args {
    int32_t nnodes;
    int32_t max_neigh;             /* power of two, 1..1024               */
    int32_t integrator;            /* PP_EULER / PP_EULER_CROMER / PP_VELOCITY_VERLET */
    int32_t precision;             /* PP_FLOAT64 / PP_MIXED                */
    int32_t nregimes;
    int32_t nbond_types;
    int32_t flags;                 /* PP_FLAG_* bits; others must be 0     */
    int32_t nodes_per_block;       /* PP_FLOAT64: warps per block, 1..8 (0 = 8) */
    int32_t variant;               /* PP_MIXED tile shape, 0..PP_MIXED_VARIANTS-1:
                                      0: 4 warps x 64 nodes per CTA,
                                      register budget for 8 resident CTAs
                                      per SM; 1: 8 warps x 128 nodes, 4
                                      CTAs/SM; 2: 8 warps x 128 nodes, 3
                                      CTAs/SM                             */
    int32_t reserved;              /* must be 0                            */
    double dt;
    double damping;
    double bond_stiffness;         /* scalar when bond_types == NULL       */
    double critical_stretch;       /* scalar when bond_types == NULL       */
    const double* bond_stiffness_table;   /* with bond_types               */
    const double* critical_stretch_table; /* with bond_types               */
    const double* plus_cs;                /* with bond_types               */
    /* static inputs, reference layouts */
    const double* r0;
    const double* vols;
    const int32_t* family;
    const int32_t* bc_types;
    const double* bc_values;
    const int32_t* fc_types;
    const double* fc_values;
    const double* densities;       /* EC / VV                              */
    const double* stiffness_corrections;  /* or NULL                       */
    const int32_t* bond_types;     /* or NULL                              */
    const double* bond_length;     /* PP_FLOAT64, optional: |r0[j] - r0[i]|
                                      per slot (nnodes, max_neigh), written
                                      by pp_bond_lengths; NULL: computed in
                                      every step (the same binary64 value) */
    /* batched independent instances (PMB only): node i uses critical
       stretch instance_s0[node_instance[i]]; NULL = one model          */
    const int32_t* node_instance;  /* (nnodes) or NULL                     */
    const double* instance_s0;     /* (ninstances)                         */
    int32_t ninstances;            /* 1..256 when node_instance != NULL    */
    int32_t reserved2;             /* must be 0                            */
    /* mutable bond state */
    int32_t* nlist;
    int32_t* regimes;              /* with bond_types                      */
    /* PP_FLOAT64 node state */
    double* u[2];
    double* ud;
    double* udd;
    double* force;
    double* body_force;
    int32_t* n_neigh;
    double* damage;
    /* PP_MIXED node state (16-byte aligned, rec 32-byte aligned) */
    float* rec[2];                 /* (nnodes) 32-byte node records        */
    float* ulo[2];
    float* vel;                    /* 2*nnodes float4                      */
    float* acc;
    float* frc;                    /* 2*nnodes float4                      */
    float* rho32;                  /* (nnodes) float4 1/density (EC / VV)  */
    float* sc32;
    int32_t* nflags;               /* (nnodes) boundary-condition flags    */
    float* umax;                   /* device word: running max of |u| (scratch) */
    int32_t* status;               /* device word: PP_STATUS_* (scratch)   */
    double pos_scale;
    double min_bond;               /* smallest |xi| over the bonds (pp_bond_extent) */
    double pos_origin[3];
    /* PP_MIXED: the tiled layout (host pointer to a struct of device
       pointers), or NULL for the untiled kernel.  With a tiling the mixed
       node state (rec, ulo, vel, acc, frc, rho32, nflags) is in internal
       order and the neighbour list, regimes, n_neigh and stiffness
       corrections are read and written through the tiling; pp_mixed_pack
       and pp_mixed_export convert from and to the reference layouts. */
    const pp_tiling* tiling;
} pp_fused_args;

/* One fused step reading state slot `parity`; magnitudes of the
 * displacement and force boundary conditions for this step by value. */
int pp_fused_step(const pp_fused_args* args, int32_t parity,
                  double displacement_bc_magnitude,
                  double force_bc_magnitude, void* stream);

/* `nsteps` fused steps starting at state slot `parity`, magnitudes read on
 * the device from disp_mags[first + k] and force_mags[first + k]
 * (k = 0..nsteps-1).  With use_graph != 0 the steps are captured in chunks
 * of `chunk` (even) launches into one CUDA graph and replayed; the step
 * index then comes from the device word *step_base (caller-allocated
 * scratch, overwritten).  The final state is in slot parity ^ (nsteps & 1). */
int pp_fused_run(const pp_fused_args* args, int32_t parity, int64_t nsteps,
                 const double* disp_mags, const double* force_mags,
                 int64_t first, int32_t use_graph, int32_t chunk,
                 int64_t* step_base, void* stream);

/* Over the bonds (i, j) of nlist (entries != -1): extent[0] = the largest
 * |r0[j][d] - r0[i][d]| over the three components d, extent[1] = the
 * smallest |r0[j] - r0[i]|; extent is two caller-allocated device doubles.
 * The caller derives pos_scale and min_bond for PP_MIXED from them. */
int pp_bond_extent(const int32_t* nlist, const double* r0, int32_t nnodes,
                   int32_t max_neigh, double* extent, void* stream);

/* Reference bond lengths for PP_FLOAT64 (pp_fused_args.bond_length):
 * length[i * max_neigh + k] = sqrt((x*x + y*y) + z*z) in binary64 with
 * (x, y, z) = r0[j] - r0[i], j = nlist[i * max_neigh + k], the value the
 * step computes for xi (peripy/cl/peridynamics.cl:65-73); 0 where j is -1.
 * A length stays valid while nlist only loses bonds (set to -1).
 * max_neigh: 1..1024 (any width: the compact rows of pp_cy_* too). */
int pp_bond_lengths(const double* r0, const int32_t* nlist, int32_t nnodes,
                    int32_t max_neigh, double* length, void* stream);

/* Builds the PP_MIXED layouts from the reference layouts: rec[parity] from
 * r0, vols (with args->pos_scale/pos_origin, which the caller chooses) and
 * u[parity], the double-float displacement slot `parity` and velocity from
 * u[parity] and
 * ud, acc from udd, sc32 from stiffness_corrections, nflags from bc_types
 * and fc_types.  Called by
 * create_buffers (peripy/integrators.py:190-254). */
int pp_mixed_pack(const pp_fused_args* args, int32_t parity, void* stream);

/* Writes the reference layouts u[parity], ud, udd, force, body_force
 * (float64) from the PP_MIXED state slot `parity`; with a tiling also the
 * -1 of every bond broken since pp_tile_rows into nlist, and regimes.
 * Called by write() (peripy/integrators.py:285-300). */
int pp_mixed_export(const pp_fused_args* args, int32_t parity, void* stream);

/* Tiled layout, first part: from the reference nlist (args->nlist,
 * args->max_neigh), args->r0, pos_scale, pos_origin and t->perm, inv,
 * tile_start, ntiles, halo_cap, writes halo, halo_count, own_off, tile_ref
 * and row_off.  A tile whose halo would exceed halo_cap, or would reach
 * 2^22 fixed-point steps or more from the tile's reference point, gets a
 * halo_count above halo_cap and no halo: the caller splits it and calls
 * again.  On return (after the stream), row_off[nnodes] is the number of
 * 16-entry blocks the rows need. */
int pp_tile_halos(const pp_fused_args* args, const pp_tiling* t, void* stream);

/* Tiled layout, second part (every halo_count <= halo_cap): writes entry,
 * slot, bond_type, regime, correction (those not NULL), the internal-order
 * copies r0, bc_values, fc_values, node_instance, and zeroes sched. */
int pp_tile_rows(const pp_fused_args* args, const pp_tiling* t, void* stream);

/* ------------------------------------------------------------------------ */
/* Neighbour families (set-up).  Replace the host KD-tree search of         */
/* Model._set_neighbour_list (peripy/model.py:536-597, sklearn KDTree       */
/* query_radius, rows padded to the CL layout at :575-585).  Two calls on   */
/* a grid of dims[0] x dims[1] x dims[2] cubic cells of edge `cell` from    */
/* the corner `lo` (host arrays of 3), covering every node, with            */
/* cell > horizon * (1 + 1e-9):                                            */
/*   pp_neighbour_cells bins the nodes: cell_start (ncells + 1 ints) and    */
/*   order (nnodes ints), device arrays the caller allocates;              */
/*   pp_neighbour_rows writes family (nnodes ints, the neighbour count of   */
/*   every node), and, when nlist is not NULL, the (nnodes, max_neigh)      */
/*   neighbour list: each row in ascending node order, padded with -1;      */
/*   rows longer than max_neigh are truncated and set *overflow (a device   */
/*   word) to 1.  Call it once with nlist = NULL to size max_neigh.         */
/* j is a neighbour of i != j when (dx*dx + dy*dy) + dz*dz <= horizon^2 in   */
/* binary64 (coords (nnodes, 3) f64 row-major on the device).               */
/* ------------------------------------------------------------------------ */

int pp_neighbour_cells(const double* coords, int32_t nnodes, const double* lo, double cell,
                       const int32_t* dims, int32_t* cell_start, int32_t* order, void* stream);

int pp_neighbour_rows(const double* coords, int32_t nnodes, double horizon, const double* lo,
                      double cell, const int32_t* dims, const int32_t* cell_start,
                      const int32_t* order, int32_t max_neigh, int32_t* nlist,
                      int32_t* family, int32_t* overflow, void* stream);

/* ------------------------------------------------------------------------ */
/* Initial crack (set-up).  Replaces peripy/create_crack.pyx:1-43, which    */
/* Model._set_neighbour_list calls (peripy/model.py:588-595): for each pair  */
/* (i, j) of crack ((npairs, 2) int32, device) in order, j is removed from  */
/* row i and then i from row j of nlist ((nnodes, max_neigh) int32, device, */
/* in/out).  A removal looks for the node among the row's first n_neigh[i]  */
/* entries; the first match is overwritten by the row's last entry, that    */
/* slot becomes -1 and n_neigh[i] ((nnodes) int32, device, in/out) drops by */
/* one; a node that is not found is skipped.  The result is that of the     */
/* sequential loop.  A negative index selects row nnodes + i, while the     */
/* node looked for is the other index as given (so a negative one is never */
/* found), as in the reference.  scratch: nnodes + 1 + 4 * npairs int32 on  */
/* the device.  An index outside [-nnodes, nnodes) sets *bad (a device      */
/* word) to 1 and leaves nlist and n_neigh unchanged; else *bad becomes 0.  */
/* ------------------------------------------------------------------------ */

int pp_create_crack(const int32_t* crack, int32_t npairs, int32_t nnodes, int32_t max_neigh,
                    int32_t* nlist, int32_t* n_neigh, int32_t* scratch, int32_t* bad,
                    void* stream);

/* ------------------------------------------------------------------------ */
/* PeriPy's CPU integrator `Euler` (peripy/integrators.py:303-459) on the   */
/* GPU: the arithmetic and the sequential semantics of the Cython module     */
/* peripy/peridynamics.pyx, bit for bit.  Layout: the compact neighbour list */
/* `Model` builds without a device context ((nnodes, max_neigh) int32, the   */
/* first n_neigh[i] entries of row i valid, max_neigh = family.max() <=      */
/* 1024, symmetric: j in row i exactly when i is in row j); coords, u,       */
/* force, bc_values, force_bc_values (nnodes, 3) f64; bc_types,              */
/* force_bc_types (nnodes, 3) int32; r = coords + u.                         */
/*   pp_cy_break_bonds: break_bonds (pyx:102-156), the result of the loop    */
/*     over nodes in ascending order: a bond (i, j), i < j, with             */
/*     !(|strain| < critical_strain) is swap-removed from row i and from row */
/*     j (vacated slots keep their stale values); n_neigh updated.           */
/*   pp_cy_bond_force: bond_force (pyx:34-99): force[i] = the sequential sum */
/*     from 0 of -f*vol[k] over lower neighbours k (ascending), +f*vol[j]    */
/*     over upper neighbours (row order), then force_bc_scale *              */
/*     force_bc_values where force_bc_types != 0.                            */
/*   pp_cy_update_displacement: update_displacement (pyx:159-184).          */
/*   pp_cy_damage: damage (pyx:5-31), (family - n_neigh) / family.          */
/* ------------------------------------------------------------------------ */

int pp_cy_break_bonds(const double* coords, const double* u, int32_t* nlist, int32_t* n_neigh,
                      int32_t nnodes, int32_t max_neigh, double critical_strain, void* stream);
int pp_cy_bond_force(const double* coords, const double* u, const int32_t* nlist,
                     const int32_t* n_neigh, const double* volume, double bond_stiffness,
                     const double* force_bc_values, const int32_t* force_bc_types,
                     double force_bc_scale, int32_t nnodes, int32_t max_neigh, double* force,
                     void* stream);
/* break_bonds then bond_force in one pass, with the results of the two
 * calls above (each bond's length and strain computed once).  bond_length
 * (optional, (nnodes, max_neigh) f64, in/out): the reference length of
 * each entry, as pp_bond_lengths writes it; read instead of computed, and
 * kept in the order of the entries as rows are edited.  NULL: computed. */
int pp_cy_break_and_force(const double* coords, const double* u, int32_t* nlist,
                          int32_t* n_neigh, const double* volume, double bond_stiffness,
                          double critical_strain, const double* force_bc_values,
                          const int32_t* force_bc_types, double force_bc_scale, int32_t nnodes,
                          int32_t max_neigh, double* force, double* bond_length, void* stream);
int pp_cy_update_displacement(double* u, const double* bc_values, const int32_t* bc_types,
                              const double* force, double bc_scale, double dt, int32_t nnodes,
                              void* stream);
int pp_cy_damage(const int32_t* n_neigh, const int32_t* family, int32_t nnodes, double* damage,
                 void* stream);
/* The precondition of the calls above, checked on the device before a
 * list is used (no counterpart in the reference, whose sequential loops
 * accept any list): *bad (one caller-allocated device word, zeroed here)
 * receives the number of entries j of a row i (among its first n_neigh[i])
 * that lie outside [0, nnodes) or whose row does not hold i exactly as
 * often as row i holds j; 0 means the list is symmetric. */
int pp_cy_check_symmetric(const int32_t* nlist, const int32_t* n_neigh, int32_t nnodes,
                          int32_t width, uint32_t* bad, void* stream);

/* ------------------------------------------------------------------------ */
/* Write-step sums.  Replace the NumPy reductions Model.simulate runs at    */
/* every write (peripy/model.py:1320-1366), so that a write needs to copy   */
/* back only u and damage (the mesh file's fields).                         */
/*   pp_pairwise_plan (host only, no CUDA call) writes the summation tree   */
/*     of NumPy's float64 sum of n contiguous elements (pairwise: leaves of */
/*     at most 128 elements summed with eight running sums, split at n / 2  */
/*     rounded down to a multiple of 8) into plan: [0] leaves, [1] inner    */
/*     nodes, [2] heights, [3] n, then leaf first elements and lengths,     */
/*     inner left and right value indices (leaves first, then inner nodes   */
/*     by height) and height offsets.  Returns the plan's length in int32;  */
/*     with plan NULL or capacity too small nothing is written; -1 when n   */
/*     is outside [0, 2^31).                                               */
/*   pp_write_sums computes, bit-identical to NumPy on the same arrays,     */
/*     sums[0..5] = np.sum of u, ud, udd, force * volume[:, None],          */
/*     body_force * volume[:, None] and damage, and for tip type t          */
/*     sums[6 + 5 t + q] = the sequential sum from 0.0 over its (node, dof) */
/*     entries of u, ud, udd, force * volume[node], body_force *            */
/*     volume[node] (q = 0..4).  A NULL ud, udd, force or body_force counts */
/*     as zeros (so do all arrays when nnodes is 0).  plan3 / plan1: device */
/*     copies of the plans of 3 nnodes and                                  */
/*     nnodes elements; scratch: 5 values3 + values1 doubles on the device. */
/* ------------------------------------------------------------------------ */

typedef struct pp_write_sums_args {
    int32_t nnodes;
    int32_t ntips;                 /* tip types                            */
    int32_t leaves3;               /* plan3[0]                             */
    int32_t values3;               /* plan3[0] + plan3[1]                  */
    int32_t leaves1;               /* plan1[0]                             */
    int32_t values1;               /* plan1[0] + plan1[1]                  */
    const double* u;               /* (nnodes, 3)                          */
    const double* ud;              /* (nnodes, 3) or NULL                  */
    const double* udd;             /* (nnodes, 3) or NULL                  */
    const double* force;           /* (nnodes, 3) or NULL                  */
    const double* body_force;      /* (nnodes, 3) or NULL                  */
    const double* damage;          /* (nnodes)                             */
    const double* volume;          /* (nnodes)                             */
    const int32_t* plan3;          /* pp_pairwise_plan(3 nnodes)           */
    const int32_t* plan1;          /* pp_pairwise_plan(nnodes)             */
    const int32_t* tip_offsets;    /* (ntips + 1) into tip_entries         */
    const int32_t* tip_entries;    /* (tip_offsets[ntips], 2) node, dof    */
    double* scratch;               /* 5 values3 + values1                  */
    double* sums;                  /* (6 + 5 ntips) out                    */
} pp_write_sums_args;

int64_t pp_pairwise_plan(int64_t n, int32_t* plan, int64_t capacity);
int pp_write_sums(const pp_write_sums_args* args, void* stream);

/* ------------------------------------------------------------------------ */
/* Stiffness correction factors (set-up).  Replaces the correction          */
/* algorithms of peripy/correction.pyx:5-277 as Model.__init__ applies them */
/* (peripy/model.py:349-375, 782-935): each selected factor multiplies the  */
/* (nnodes, max_neigh) f64 array `corrections` in place, in the order       */
/* micromodulus, volume, surface.  Rows hold their n_neigh[i] bonds first   */
/* (no repeated neighbour); other slots are left as they are.              */
/*   micromodulus_function 0: conical, (h - l0)/h within h = micromodulus_  */
/*     horizon; -1: none                                                    */
/*   volume_correction 0: partial volume, 1 for l0 <= H - R, (H + R - l0) / */
/*     (2 R) up to H + R, else 0, with H = vc_horizon, R = vc_node_radius;  */
/*     -1: none                                                            */
/*   surface_correction 1: 2 family_volume_bulk / (V_i + V_j) with V the    */
/*     summed volumes of a node's bonds; 0: the same with V = n_neigh *     */
/*     average_volume; -1: none.  family_volume: (nnodes) f64 scratch.      */
/* l0 = |r0[j] - r0[i]| in binary64.                                        */
/* ------------------------------------------------------------------------ */

typedef struct pp_corrections_args {
    int32_t nnodes;
    int32_t max_neigh;
    int32_t micromodulus_function;
    int32_t volume_correction;
    int32_t surface_correction;
    int32_t reserved;              /* must be 0                            */
    double micromodulus_horizon;
    double vc_horizon;
    double vc_node_radius;
    double family_volume_bulk;
    double average_volume;
    const double* r0;              /* (nnodes, 3)                          */
    const double* volume;          /* (nnodes)                             */
    const int32_t* nlist;          /* (nnodes, max_neigh)                  */
    const int32_t* n_neigh;        /* (nnodes)                             */
    double* corrections;           /* (nnodes, max_neigh), in/out          */
    double* family_volume;         /* (nnodes) scratch (surface correction) */
} pp_corrections_args;

int pp_stiffness_corrections(const pp_corrections_args* args, void* stream);

/* ------------------------------------------------------------------------ */
/* Adjoint of the Euler step (gradients of a displacement loss).            */
/* No counterpart in the reference: PeriPy has no gradients.  The forward  */
/* step is pp_fused_step with PP_FLOAT64, PP_EULER, stiffness corrections   */
/* = per-bond stiffness k_b, bond_stiffness = 1 and critical_stretch =      */
/* +inf (the bond set is frozen); this is the reverse of that step.         */
/* ------------------------------------------------------------------------ */

typedef struct pp_adjoint_args {
    int32_t nnodes;
    int32_t max_neigh;             /* power of two, 1..1024               */
    double dt;
    const double* r0;              /* (nnodes,3)                           */
    const double* vols;            /* (nnodes)                             */
    const int32_t* nlist;          /* (nnodes,max_neigh), -1 = no bond     */
    const int32_t* partner;        /* from pp_partner_slots                */
    const int32_t* bc_types;       /* (nnodes,3): nonzero = prescribed DOF */
    const double* stiffness;       /* (nnodes,max_neigh) per-bond k_b      */
} pp_adjoint_args;

/* partner[i][s] = the slot of i in row nlist[i][s] (or -1): where the
 * reverse bond's data lives. */
int pp_partner_slots(const int32_t* nlist, int32_t nnodes, int32_t max_neigh,
                     int32_t* partner, void* stream);

/* break_step[g] = t for every slot g with nlist[g] == -1 and
 * break_step[g] > t: called after forward step t, it records the first step
 * at which each bond is broken (initialise break_step to INT32_MAX). */
int pp_mark_breaks(const int32_t* nlist, int32_t* break_step, int64_t nslots,
                   int32_t t, void* stream);

/* nlist_t[g] = break_step[g] > t ? nlist0[g] : -1: the bond set in force
 * during step t, frozen for recomputation and the reverse step. */
int pp_bonds_at_step(const int32_t* nlist0, const int32_t* break_step,
                     int64_t nslots, int32_t t, int32_t* nlist_t, void* stream);

/* One reverse step: from lam_next = dL/du_{t+1} and the state u = u_t,
 * writes lam = dL/du_t and adds dL/dk_b of this step to grad_k
 * ((nnodes,max_neigh)). */
int pp_adjoint_backward(const pp_adjoint_args* args, const double* u,
                        const double* lam_next, double* lam, double* grad_k,
                        void* stream);

/* ------------------------------------------------------------------------ */
/* Fused steps without any device allocation.                               */
/* ------------------------------------------------------------------------ */

/* Largest nsteps accepted by pp_fused_run_static. */
#define PP_STATIC_MAX_STEPS         65536

/* No counterpart in the reference: an addition for callers that cannot
 * allocate device memory themselves -- for instance code running inside a
 * host runtime whose device memory is pre-reserved and handed out only as
 * the simulation arrays, or a caller that must not change the device
 * memory footprint between set-up and the time loop.  pp_fused_run needs a
 * caller-allocated device copy of the magnitude schedules and a step-index
 * word, and the mixed-precision step needs two caller-allocated device
 * words; this entry point needs none of them.
 *
 * Same steps as pp_fused_run(args, parity, nsteps, ...) with direct launches
 * (no CUDA graph), except that disp_mags[k] and force_mags[k] are read from
 * HOST memory (k = 0..nsteps-1) and copied into a file-scope device array
 * of the library (1 MB: 2 * PP_STATIC_MAX_STEPS doubles plus two words),
 * which every GPU that loads the library holds until the process exits.
 * For PP_MIXED, args->umax and args->status are ignored: the call keeps
 * those words in the same array, clears the status word and recomputes the
 * running max |u| from the state at its start; pp_static_status() reads the
 * status word back.  nsteps > PP_STATIC_MAX_STEPS returns
 * PP_ERROR_TOO_LARGE.  It calls no cudaMalloc, cudaFree or other allocating
 * routine.
 *
 * The schedule is copied with cudaMemcpyAsync on `stream`.  From pageable
 * host memory the copy completes before the call returns; from page-locked
 * (pinned or registered) memory it is truly asynchronous, so the caller
 * must keep disp_mags[0..nsteps) and force_mags[0..nsteps) allocated and
 * unchanged until the stream has executed the call.  A pageable source
 * cannot be captured into a CUDA graph; make no claim here beyond that.
 *
 * The first call in each CUDA context looks up the array's device address
 * (cudaGetSymbolAddress, with that device current) and caches it together
 * with the context's unique ID, so after a device reset or a re-created
 * primary context the next call looks it up again; make that first call
 * before any stream capture.  All calls share the one array: calls whose
 * work overlaps on the GPU (different streams, or host threads) race on it
 * and must be serialised by the caller. */
int pp_fused_run_static(const pp_fused_args* args, int32_t parity,
                        int64_t nsteps, const double* disp_mags,
                        const double* force_mags, void* stream);

/* ------------------------------------------------------------------------ */
/* Host memory.  Page-lock (cudaHostRegister) and release a caller host     */
/* array, used for the device-to-host copies of write().  No counterpart in */
/* the reference (pyopencl copies into pageable arrays).  A failed          */
/* registration returns PP_ERROR_CUDA and leaves no pending error in the   */
/* library's runtime; the array can still be copied as pageable memory.    */
/* ------------------------------------------------------------------------ */
int pp_host_register(void* ptr, size_t bytes);
int pp_host_unregister(void* ptr);

/* Copies the status word of the last pp_fused_run_static call on `stream`
 * (PP_STATUS_*) to *status (host memory) and waits for the stream.  No
 * counterpart in the reference. */
int pp_static_status(int32_t* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PP_GB300_H */
