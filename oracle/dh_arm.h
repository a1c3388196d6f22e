/*
 * ORACLE (test infrastructure only): definition of the serial-arm sphere checker used by the
 * 7-DoF arm workloads. OMPL has no counterpart in its own sources (its arm checking lives in the
 * absent VAMP submodule), so this header IS the definition; the CPU restatement and the build of
 * OMPL's sources both include it, and the GPU FP64 path reproduces it operation for operation.
 * Compile with -ffp-contract=off.
 */
#ifndef GBOMPL_ORACLE_DH_ARM_H
#define GBOMPL_ORACLE_DH_ARM_H
#include "oracle_api.h"
#include <cmath>
#include <vector>

namespace gbompl_oracle
{
/* Serial arm with standard Denavit-Hartenberg rows, covered by spheres (no counterpart in OMPL:
 * the reference's arm checking lives in the absent VAMP submodule). Definition, in FP64 and in
 * exactly this operation order:
 *   frame 0 = identity. For joint i: c = cos(q_i), s = sin(q_i); (ca, sa) = (1,0), (0,1), (0,-1)
 *   for alpha_code 0, +1, -1. A = [[c, -s*ca, s*sa], [s, c*ca, -c*sa], [0, sa, ca]], pA = (a*c, a*s, d).
 *   R' = R*A with R'[r][k] = (R[r][0]*A[0][k] + R[r][1]*A[1][k]) + R[r][2]*A[2][k];
 *   p' = ((R[r][0]*pA[0] + R[r][1]*pA[1]) + R[r][2]*pA[2]) + p[r].
 *   Link i spans p_i -> p_{i+1}; its spheres sit at p_i + f*(p_{i+1} - p_i), f = (k + 0.5)/spheres_per_link.
 *   A robot sphere (centre c, radius rs) hits world sphere (o, ro) iff
 *   (dx*dx + dy*dy) + dz*dz < (rs + ro)*(rs + ro) with d = c - o (boxes: dh_pair_hits); the state is
 *   valid iff nothing hits. */
inline void dh_sphere_centres(const ora_checker *c, const double *q, double *centres /* n_joints*spl*3 */)
{
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double p[3] = {0, 0, 0};
    const int spl = c->spheres_per_link;
    for (int i = 0; i < c->n_joints; ++i)
    {
        const double a = c->dh[3 * i + 0], d = c->dh[3 * i + 1];
        const int code = (int)c->dh[3 * i + 2];
        const double ca = code == 0 ? 1.0 : 0.0;
        const double sa = code == 0 ? 0.0 : (code > 0 ? 1.0 : -1.0);
        const double cq = std::cos(q[i]), sq = std::sin(q[i]);
        const double A[3][3] = {{cq, -sq * ca, sq * sa}, {sq, cq * ca, -cq * sa}, {0.0, sa, ca}};
        const double pA[3] = {a * cq, a * sq, d};
        double Rn[3][3], pn[3];
        for (int r = 0; r < 3; ++r)
        {
            for (int k = 0; k < 3; ++k)
                Rn[r][k] = (R[r][0] * A[0][k] + R[r][1] * A[1][k]) + R[r][2] * A[2][k];
            pn[r] = ((R[r][0] * pA[0] + R[r][1] * pA[1]) + R[r][2] * pA[2]) + p[r];
        }
        for (int k = 0; k < spl; ++k)
        {
            const double f = ((double)k + 0.5) / (double)spl;
            double *ctr = centres + 3 * (i * spl + k);
            for (int r = 0; r < 3; ++r)
                ctr[r] = p[r] + f * (pn[r] - p[r]);
        }
        for (int r = 0; r < 3; ++r)
        {
            p[r] = pn[r];
            for (int k = 0; k < 3; ++k)
                R[r][k] = Rn[r][k];
        }
    }
}

/* Narrow phase of one robot sphere (centre p, radius rs) against world obstacle o.
 *   sphere (x, y, z, r): hit iff (dx*dx + dy*dy) + dz*dz < (rs + r)*(rs + r), d = p - o;
 *   box (cx, cy, cz, hx, hy, hz), kind ORA_CHECK_DH_BOXES: per axis g = fabs(p - c) - h, g = 0 when
 *   g <= 0 (g > 0 ? g : 0), hit iff (gx*gx + gy*gy) + gz*gz < rs*rs (the squared distance of p from
 *   the box is below rs^2). */
inline bool dh_pair_hits(const double *p, const double *o, double rs, bool boxes)
{
    if (boxes)
    {
        double gx = std::fabs(p[0] - o[0]) - o[3];
        double gy = std::fabs(p[1] - o[1]) - o[4];
        double gz = std::fabs(p[2] - o[2]) - o[5];
        gx = gx > 0.0 ? gx : 0.0;
        gy = gy > 0.0 ? gy : 0.0;
        gz = gz > 0.0 ? gz : 0.0;
        return (gx * gx + gy * gy) + gz * gz < rs * rs;
    }
    double dx = p[0] - o[0];
    double dy = p[1] - o[1];
    double dz = p[2] - o[2];
    double rr = rs + o[3];
    return (dx * dx + dy * dy) + dz * dz < rr * rr;
}

inline bool dh_valid(const ora_checker *c, const double *q)
{
    const int ns = c->n_joints * c->spheres_per_link;
    std::vector<double> ctr(3 * (size_t)ns);
    dh_sphere_centres(c, q, ctr.data());
    const bool boxes = c->kind == ORA_CHECK_DH_BOXES;
    const int stride = boxes ? 6 : 4;
    for (int s = 0; s < ns; ++s)
        for (long j = 0; j < c->n_obstacles; ++j)
            if (dh_pair_hits(&ctr[3 * s], c->obstacles + stride * j, c->sphere_radius, boxes))
                return false;
    return true;
}

}  // namespace gbompl_oracle
#endif
