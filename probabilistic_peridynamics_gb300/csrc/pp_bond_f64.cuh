// pp_bond_f64.cuh -- binary64 per-bond arithmetic shared by the plain and
// fused FP64 kernels.
//
// Restates the per-work-item body of bond_force1..4
// (peripy/cl/peridynamics.cl:61-102, 193-233, 323-385, 474-536) with exact
// round-to-nearest intrinsics and the reference association order:
//   xi   = r0[j] - r0[i]                           (:65-67)
//   xe   = (u[j] - u[i]) + xi                      (:69-71)
//   |xi| = sqrt((x*x + y*y) + z*z), |xe| likewise  (:73-74)
//   s    = (|xe| - |xi|) / |xi|                    (:75)
//   PMB:      intact iff s < s0, f = (s*k)[*corr]*vol[j]            (:78-83, :214)
//   n-linear: regime moves by at most one, breaks at r >= nregimes,
//             f = ((s*k[r] + c[r])[*corr])*vol[j]                     (:345-373, :524)
//   force component = f * (xe / |xe|)                                (:79-87)
#pragma once

#include "pp_common.cuh"

namespace pp {

struct F64Bond {
    const double* r0;
    const double* u;
    const double* vols;
    int32_t* nlist;
    const double* sc;         // stiffness corrections or nullptr
    const int32_t* btypes;    // bond types or nullptr
    int32_t* regimes;
    const double* ktab;
    const double* stab;
    const double* ctab;
    const double* xi_len;     // per-slot |xi| (pp_bond_lengths) or nullptr
    double k;
    double s0;
    int nregimes;
};

// Contribution of slot `gid` of node i.  Breaks the bond / moves its regime
// in place exactly as the reference kernel does; counts intact bonds.
template <bool CORR, bool TYPES>
__device__ __forceinline__ d3 f64_slot(const F64Bond& b, int64_t gid, d3 ri, d3 ui,
                                       int& intact) {
    const int j = b.nlist[gid];
    if (j == -1) return d3_zero();
    const double* rj = b.r0 + 3 * (int64_t)j;
    const double* uj = b.u + 3 * (int64_t)j;
    const double xi_x = dsub(rj[0], ri.x);
    const double xi_y = dsub(rj[1], ri.y);
    const double xi_z = dsub(rj[2], ri.z);
    const double xe_x = dadd(dsub(uj[0], ui.x), xi_x);
    const double xe_y = dadd(dsub(uj[1], ui.y), xi_y);
    const double xe_z = dadd(dsub(uj[2], ui.z), xi_z);
    // |xi| never changes: read it when cached (the same binary64 value)
    const double xi = b.xi_len ? b.xi_len[gid]
                               : dsqrt(dadd(dadd(dmul(xi_x, xi_x), dmul(xi_y, xi_y)),
                                            dmul(xi_z, xi_z)));
    const double y = dsqrt(dadd(dadd(dmul(xe_x, xe_x), dmul(xe_y, xe_y)), dmul(xe_z, xe_z)));
    const double s = ddiv(dsub(y, xi), xi);
    double f;
    if constexpr (!TYPES) {
        if (!(s < b.s0)) {
            b.nlist[gid] = -1;
            return d3_zero();
        }
        f = dmul(s, b.k);
        if constexpr (CORR) f = dmul(f, b.sc[gid]);
        f = dmul(f, b.vols[j]);
    } else {
        const int nr = b.nregimes;
        const int base = b.btypes[gid] * nr;
        int r = b.regimes[gid];
        // A valid bond always has 0 <= r < nregimes; clamp the table reads
        // so that a malformed regimes array cannot read out of bounds.
        const int rc = r < 0 ? 0 : (r >= nr ? nr - 1 : r);
        if (s < b.stab[base + rc]) {
            if (r > 0 && rc > 0) {
                if (s < b.stab[base + rc - 1]) {
                    r -= 1;
                    b.regimes[gid] = r;
                }
            }
        } else {
            r += 1;
            b.regimes[gid] = r;
        }
        if (r >= nr) {
            b.nlist[gid] = -1;
            return d3_zero();
        }
        const int rr = r < 0 ? 0 : r;
        f = dadd(dmul(s, b.ktab[base + rr]), b.ctab[base + rr]);
        if constexpr (CORR) f = dmul(f, b.sc[gid]);
        f = dmul(f, b.vols[j]);
    }
    intact += 1;
    return d3{dmul(f, ddiv(xe_x, y)), dmul(f, ddiv(xe_y, y)), dmul(f, ddiv(xe_z, y))};
}

// Euler update of one DOF (peripy/cl/euler.cl:23).
__device__ __forceinline__ double euler_u(double u, double f, int bct, double bcv,
                                          double bc_scale, double dt) {
    return bct == 0 ? dadd(u, dmul(dt, f)) : dmul(bc_scale, bcv);
}

// Euler-Cromer update of one DOF (peripy/cl/euler_cromer.cl:55-58).
__device__ __forceinline__ double euler_cromer_u(double u, double& ud, double& udd, double f,
                                                 int bct, double bcv, double rho,
                                                 double bc_scale, double damping,
                                                 double dt) {
    const double uddi = ddiv(dsub(f, dmul(damping, ud)), rho);
    udd = uddi;
    ud = dadd(ud, dmul(uddi, dt));
    return bct == 0 ? dadd(u, dmul(dt, ud)) : dmul(bc_scale, bcv);
}

// Velocity-Verlet update of one DOF (peripy/cl/velocity_verlet.cl:90-94).
__device__ __forceinline__ double velocity_verlet_u(double u, double& ud, double& udd,
                                                    double f, int bct, double bcv,
                                                    double rho, double bc_scale,
                                                    double damping, double dt) {
    const double half = ddiv(dt, 2.0);
    const double ud1 = dadd(ud, dmul(half, udd));
    const double udd1 = ddiv(dsub(f, dmul(damping, ud1)), rho);
    ud = dadd(ud1, dmul(half, udd1));
    udd = udd1;
    return bct == 0 ? dadd(u, dmul(dt, dadd(ud, dmul(half, udd1)))) : dmul(bc_scale, bcv);
}

// Force with the force boundary condition (peridynamics.cl:127-129).
__device__ __forceinline__ double force_with_bc(double body, int fct, double fcv,
                                                double fc_scale) {
    return fct == 0 ? body : dadd(body, dmul(fc_scale, fcv));
}

// Damage of one node (peridynamics.cl:606-608).
__device__ __forceinline__ double damage_of(int intact, int family) {
    return dsub(1.0, ddiv((double)intact, (double)family));
}

}  // namespace pp
