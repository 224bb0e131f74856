/*
 * pp_oracle.c -- C restatement of PeriPy's OpenCL time step
 * (TEST INFRASTRUCTURE: the checker and the port-kind CPU baseline; the
 * product never links or calls it).
 *
 * Same arithmetic, operation order and work-group tree reduction order as
 * oracle/cl_step.py, which follows:
 *   pp_oracle_bond_force  peripy/cl/peridynamics.cl:4-565 (bond_force1..4)
 *   pp_oracle_damage      peripy/cl/peridynamics.cl:568-610
 *   pp_oracle_update      peripy/cl/euler.cl:21-23, euler_cromer.cl:53-58,
 *                         velocity_verlet.cl:88-94
 * Compile with -ffp-contract=off (no fused multiply-add) and without
 * -ffast-math so every binary64 operation rounds as written.  Nodes are
 * independent within a pass, so the node loop runs under OpenMP; each node's
 * slots are evaluated and reduced in a fixed order, so results do not depend
 * on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 1024

static void tree(double* c, int L) {
    for (int w = L / 2; w >= 1; w /= 2)
        for (int l = 0; l < w; ++l) c[l] = c[l] + c[l + w];
}

/* Returns 0, or 1 when max_neigh is not a power of two <= 1024. */
int pp_oracle_bond_force(int n, int L, const double* u, const double* r0,
                         const double* vols, int32_t* nlist,
                         const int32_t* fct, const double* fcv,
                         double fc_scale, double k, double s0,
                         const double* sc, const int32_t* bt,
                         int32_t* regimes, const double* ktab,
                         const double* stab, const double* ctab,
                         int nregimes, double* force, double* body_force) {
    if (L < 1 || L > MAXL || (L & (L - 1))) return 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double cx[MAXL], cy[MAXL], cz[MAXL];
        for (int l = 0; l < L; ++l) {
            const int64_t gid = (int64_t)i * L + l;
            const int j = nlist[gid];
            cx[l] = cy[l] = cz[l] = 0.0;
            if (j == -1) continue;
            const double xi_x = r0[3 * (int64_t)j] - r0[3 * (int64_t)i];
            const double xi_y = r0[3 * (int64_t)j + 1] - r0[3 * (int64_t)i + 1];
            const double xi_z = r0[3 * (int64_t)j + 2] - r0[3 * (int64_t)i + 2];
            const double xe_x = u[3 * (int64_t)j] - u[3 * (int64_t)i] + xi_x;
            const double xe_y = u[3 * (int64_t)j + 1] - u[3 * (int64_t)i + 1] + xi_y;
            const double xe_z = u[3 * (int64_t)j + 2] - u[3 * (int64_t)i + 2] + xi_z;
            const double xi = sqrt(xi_x * xi_x + xi_y * xi_y + xi_z * xi_z);
            const double y = sqrt(xe_x * xe_x + xe_y * xe_y + xe_z * xe_z);
            const double s = (y - xi) / xi;
            double f;
            if (!bt) {
                if (!(s < s0)) {
                    nlist[gid] = -1;
                    continue;
                }
                f = s * k;
                if (sc) f = f * sc[gid];
                f = f * vols[j];
            } else {
                const int nr = nregimes;
                const int base = bt[gid] * nr;
                int r = regimes[gid];
                const int rc = r < 0 ? 0 : (r >= nr ? nr - 1 : r);
                if (s < stab[base + rc]) {
                    if (r > 0 && rc > 0 && s < stab[base + rc - 1]) {
                        r -= 1;
                        regimes[gid] = r;
                    }
                } else {
                    r += 1;
                    regimes[gid] = r;
                }
                if (r >= nr) {
                    nlist[gid] = -1;
                    continue;
                }
                const int rr = r < 0 ? 0 : r;
                f = s * ktab[base + rr] + ctab[base + rr];
                if (sc) f = f * sc[gid];
                f = f * vols[j];
            }
            cx[l] = f * (xe_x / y);
            cy[l] = f * (xe_y / y);
            cz[l] = f * (xe_z / y);
        }
        tree(cx, L);
        tree(cy, L);
        tree(cz, L);
        const double b[3] = {cx[0], cy[0], cz[0]};
        for (int d = 0; d < 3; ++d) {
            const int64_t o = 3 * (int64_t)i + d;
            body_force[o] = b[d];
            force[o] = fct[o] == 0 ? b[d] : b[d] + fc_scale * fcv[o];
        }
    }
    return 0;
}

void pp_oracle_damage(int n, int L, const int32_t* nlist,
                      const int32_t* family, int32_t* n_neigh,
                      double* damage) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        int count = 0;
        for (int l = 0; l < L; ++l) count += nlist[(int64_t)i * L + l] != -1;
        n_neigh[i] = count;
        damage[i] = 1.00 - (double)count / (double)family[i];
    }
}

/* kind: 0 Euler, 1 Euler-Cromer, 2 Velocity-Verlet. */
void pp_oracle_update(int kind, int64_t ndof, const double* force, double* u,
                      double* ud, double* udd, const int32_t* bc_types,
                      const double* bc_values, const double* densities,
                      double bc_scale, double damping, double dt) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < ndof; ++i) {
        if (kind == 0) {
            u[i] = bc_types[i] == 0 ? u[i] + dt * force[i] : bc_scale * bc_values[i];
        } else if (kind == 1) {
            const double uddi = (force[i] - damping * ud[i]) / densities[i];
            udd[i] = uddi;
            ud[i] += uddi * dt;
            u[i] = bc_types[i] == 0 ? u[i] + dt * ud[i] : bc_scale * bc_values[i];
        } else {
            const double ud1 = ud[i] + (dt / 2) * udd[i];
            const double udd1 = (force[i] - damping * ud1) / densities[i];
            ud[i] = ud1 + (dt / 2) * udd1;
            udd[i] = udd1;
            u[i] = bc_types[i] == 0 ? u[i] + dt * (ud[i] + (dt / 2) * udd1)
                                    : bc_scale * bc_values[i];
        }
    }
}
