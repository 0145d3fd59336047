// Analytic magnets, FP64, with the reference's operation order and no fused multiply-adds,
// so that boundary decisions and values match the CPU code.  16-double records:
//   QS / Q   origin, XI, YI, ZI, length, gradient, second gradient, aperture radius
//            (magnets.py:637-668 field, :726-748 record; a Q has no second gradient, :762-801)
//   straight dipole (LocalUniformMagnet, magnets.py:440-481): the same frame, -length, field,
//            0, aperture radius -- a negative length marks this kind; field = YI * field inside
//            the cylinder of the aperture radius for 0 <= z <= length
//   uniform  (UniformMagnet, magnets.py:417-437): length -inf, field YI * q[13] everywhere.
// Points go to the local frame as local_coordinate_system.py:60-74 does.
#pragma once

__device__ __forceinline__ void qs_field_add(const double *__restrict__ q, double px, double py, double pz,
                                             double &bx, double &by, double &bz) {
    if (q[12] < 0.0 && isinf(q[12])) {   // uniform everywhere
        bx = __dadd_rn(bx, __dmul_rn(q[6], q[13]));
        by = __dadd_rn(by, __dmul_rn(q[7], q[13]));
        bz = __dadd_rn(bz, __dmul_rn(q[8], q[13]));
        return;
    }
    const double dx = __dadd_rn(px, -q[0]), dy = __dadd_rn(py, -q[1]), dz = __dadd_rn(pz, -q[2]);
    const double x = __dadd_rn(__dadd_rn(__dmul_rn(q[3], dx), __dmul_rn(q[4], dy)), __dmul_rn(q[5], dz));
    const double y = __dadd_rn(__dadd_rn(__dmul_rn(q[6], dx), __dmul_rn(q[7], dy)), __dmul_rn(q[8], dz));
    const double z = __dadd_rn(__dadd_rn(__dmul_rn(q[9], dx), __dmul_rn(q[10], dy)), __dmul_rn(q[11], dz));
    if (q[12] < 0.0) {                   // straight dipole of length -q[12]
        if (z < 0.0 || z > -q[12]) return;
        const double a = q[15];
        if (fabs(x) > a || fabs(y) > a || sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))) > a) return;
        bx = __dadd_rn(bx, __dmul_rn(q[6], q[13]));
        by = __dadd_rn(by, __dmul_rn(q[7], q[13]));
        bz = __dadd_rn(bz, __dmul_rn(q[8], q[13]));
        return;
    }
    if (z < 0.0 || z > q[12]) return;
    const double a = q[15];
    if (fabs(x) > a || fabs(y) > a || sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))) > a) return;
    const double g = q[13], s = q[14];
    const double lbx = __dadd_rn(__dmul_rn(g, y), __dmul_rn(s, __dmul_rn(x, y)));
    const double lby = __dadd_rn(__dmul_rn(g, x),
                                 __dmul_rn(__dmul_rn(0.5, s), __dadd_rn(__dmul_rn(x, x), -__dmul_rn(y, y))));
    bx = __dadd_rn(bx, __dadd_rn(__dmul_rn(q[3], lbx), __dmul_rn(q[6], lby)));
    by = __dadd_rn(by, __dadd_rn(__dmul_rn(q[4], lbx), __dmul_rn(q[7], lby)));
    bz = __dadd_rn(bz, __dadd_rn(__dmul_rn(q[5], lbx), __dmul_rn(q[8], lby)));
}
