/* Generated by pentrack_gb300/csrc/gen_constants.py -- do not edit.
 * PENTrack's physical constants (src/globals.cpp:13-32), evaluated in x86
 * 80-bit long double as the reference does, then rounded once to double. */
#ifndef PT_CONSTANTS_H
#define PT_CONSTANTS_H

#define PT_PI 0x1.921fb54442d18p+1 /* 3.141592653589793 */
#define PT_ELE_E 0x1.7a4da04a6daf5p-63 /* 1.602176487e-19 */
#define PT_GRAVCONST 0x1.39d013a92a305p+3 /* 9.80665 */
#define PT_C0 0x1.1de784a000000p+28 /* 299792458.0 */
#define PT_HBAR 0x1.185a7f04cca12p-113 /* 1.05457266e-34 */
#define PT_M_N 0x1.673302a9f27acp-27 /* 1.0454074345680994e-08 */
#define PT_M_P 0x1.66b46eac7abf4p-27 /* 1.0439684083317845e-08 */
#define PT_M_E 0x1.901732cb621c3p-38 /* 5.685629656853153e-12 */
#define PT_MU_N_SI -0x1.7ec4036197f3ap-87 /* -9.6623641e-27 */
#define PT_GAMMA_N -0x1.5d842a2000000p+27 /* -183247185.0 */

/* Per-species derived constants: charge q [C], mass m [eV/c^2], magnetic moment mu [J/T],
 * gyromagnetic ratio [1/(T s)], mass in kg (m*e), gravity force -g*m*e [N],
 * mu/e [eV/T] and q/e, each computed in long double and rounded once. */
#define PT_NEUTRON_Q 0x0.0p+0
#define PT_NEUTRON_M 0x1.673302a9f27acp-27
#define PT_NEUTRON_MU -0x1.7ec4036197f3ap-87
#define PT_NEUTRON_GAMMA -0x1.5d842a2000000p+27
#define PT_NEUTRON_MKG 0x1.09671e9786bb7p-89
#define PT_NEUTRON_INV_MKG 0x1.eddc5270bb842p+88
#define PT_NEUTRON_FGRAV -0x1.4556cc9226ee2p-86
#define PT_NEUTRON_MU_OVER_E -0x1.03050f5bc549dp-24
#define PT_NEUTRON_Q_OVER_E 0x0.0p+0
#define PT_NEUTRON_MC2 0x1.c005090daa164p+29
#define PT_NEUTRON_MG 0x1.b851534a189ebp-24
#define PT_PROTON_Q 0x1.7a4da04a6daf5p-63
#define PT_PROTON_M 0x1.66b46eac7abf4p-27
#define PT_PROTON_MU 0x0.0p+0
#define PT_PROTON_GAMMA 0x0.0p+0
#define PT_PROTON_MKG 0x1.090998248311dp-89
#define PT_PROTON_INV_MKG 0x1.ee8a97e0eddcbp+88
#define PT_PROTON_FGRAV -0x1.44e4272b1b390p-86
#define PT_PROTON_MU_OVER_E 0x0.0p+0
#define PT_PROTON_Q_OVER_E 0x1.0000000000000p+0
#define PT_PROTON_MC2 0x1.bf67286b68167p+29
#define PT_PROTON_MG 0x1.b7b629773aa8cp-24
#define PT_ELECTRON_Q -0x1.7a4da04a6daf5p-63
#define PT_ELECTRON_M 0x1.901732cb621c3p-38
#define PT_ELECTRON_MU 0x0.0p+0
#define PT_ELECTRON_GAMMA 0x0.0p+0
#define PT_ELECTRON_MKG 0x1.279dc93eb3f4ep-100
#define PT_ELECTRON_INV_MKG 0x1.bb62af3b66c07p+99
#define PT_ELECTRON_FGRAV -0x1.6a6031f53ac9ep-97
#define PT_ELECTRON_MU_OVER_E 0x0.0p+0
#define PT_ELECTRON_Q_OVER_E -0x1.0000000000000p+0
#define PT_ELECTRON_MC2 0x1.f305ba3af1994p+18
#define PT_ELECTRON_MG 0x1.ea718eae0a393p-35

#define PT_C0_SQ 0x1.3f4d4eacdd756p+56
#define PT_INV_C0_SQ 0x1.9a7ed39e826dap-57
#define PT_MAX_TRACK_DEVIATION 0x1.0624dd2f1a9fcp-10 /* 0.001 m, include/particle.h:20 */
#define PT_REFLECT_TOLERANCE 1e-8 /* include/trianglemesh.h:39 */

#endif
