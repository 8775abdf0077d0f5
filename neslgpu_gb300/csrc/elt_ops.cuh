// elt_ops.cuh -- the element functions of the elementwise CVL maps
// (nesl/cvl/serial/elwise.c:192-298), one struct per (operation, type)
// with a static device f().  C semantics exactly: int + - * wrap (done in
// unsigned), / and % truncate, shift counts are taken modulo 32, booleans
// are 0/1 ints, rou is (int)(x + 0.5), floor/ceil/trunc convert with (int);
// transcendentals call the CUDA double-precision math library.  Used by
// elementwise.cu and by the generated fused super-op kernels.
#pragma once

namespace gcvl {

#define F2(NAME, TI, TO, EXPR) \
  struct NAME { __device__ static TO f(TI x, TI y) { return (TO)(EXPR); } };
#define F1(NAME, TI, TO, EXPR) \
  struct NAME { __device__ static TO f(TI x) { return (TO)(EXPR); } };

F2(f_max_z, int, int, x > y ? x : y)
F2(f_max_d, double, double, x > y ? x : y)
F2(f_min_z, int, int, x < y ? x : y)
F2(f_min_d, double, double, x < y ? x : y)
F2(f_add_z, int, int, (unsigned)x + (unsigned)y)
F2(f_add_d, double, double, __dadd_rn(x, y))
F2(f_sub_z, int, int, (unsigned)x - (unsigned)y)
F2(f_sub_d, double, double, __dsub_rn(x, y))
F2(f_mul_z, int, int, (unsigned)x * (unsigned)y)
F2(f_mul_d, double, double, __dmul_rn(x, y))
F2(f_div_z, int, int, x / y)
F2(f_div_d, double, double, __ddiv_rn(x, y))
F2(f_grt_z, int, int, x > y)
F2(f_grt_d, double, int, x > y)
F2(f_les_z, int, int, x < y)
F2(f_les_d, double, int, x < y)
F2(f_geq_z, int, int, x >= y)
F2(f_geq_d, double, int, x >= y)
F2(f_leq_z, int, int, x <= y)
F2(f_leq_d, double, int, x <= y)
F2(f_lsh_z, int, int, (unsigned)x << (y & 31))
F2(f_rsh_z, int, int, x >> (y & 31))
F2(f_mod_z, int, int, x % y)
F2(f_eql_z, int, int, x == y)
F2(f_eql_d, double, int, x == y)
F2(f_neq_z, int, int, x != y)
F2(f_neq_d, double, int, x != y)
F2(f_xor_b, int, int, x ^ y)
F2(f_ior_b, int, int, x || y)
F2(f_and_b, int, int, x && y)
F2(f_ior_z, int, int, x | y)
F2(f_and_z, int, int, x & y)
F2(f_xor_z, int, int, x ^ y)
F1(f_not_b, int, int, !x)
F1(f_not_z, int, int, ~x)
F1(f_int_d, double, int, (int)x)
F1(f_int_b, int, int, x)
F1(f_dbl_z, int, double, (double)x)
F1(f_boo_z, int, int, x != 0)
F1(f_flr_d, double, int, (int)floor(x))
F1(f_cei_d, double, int, (int)ceil(x))
F1(f_trn_d, double, int, (int)x)
F1(f_rou_d, double, int, (int)__dadd_rn(x, 0.5))
F1(f_exp_d, double, double, exp(x))
F1(f_log_d, double, double, log(x))
F1(f_sqt_d, double, double, sqrt(x))
F1(f_sin_d, double, double, sin(x))
F1(f_cos_d, double, double, cos(x))
F1(f_tan_d, double, double, tan(x))
F1(f_asn_d, double, double, asin(x))
F1(f_acs_d, double, double, acos(x))
F1(f_atn_d, double, double, atan(x))
F1(f_snh_d, double, double, sinh(x))
F1(f_csh_d, double, double, cosh(x))
F1(f_tnh_d, double, double, tanh(x))
F1(f_cpy_z, int, int, x)
F1(f_cpy_d, double, double, x)


}  // namespace gcvl
