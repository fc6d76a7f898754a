// Physical constants of the MOLOCH step, host and device.
// Values and the expressions that derive them are those of the reference's
// mod_constants.F90 (line numbers below); they must agree to the last bit
// with the FP64 reference, so derived constants are written as the same
// expressions and folded by the compiler in IEEE double precision.
#pragma once

namespace moloch {

constexpr double kEgrav = 9.80665;                         // :81
constexpr double kNavgdr = 6.02214076e23;                  // :90
constexpr double kBoltzk = 1.3806490e-23;                  // :88
constexpr double kAmd = 28.96454;                          // :103
constexpr double kAmw = 18.01528;                          // :105
constexpr double kRgasmol = kNavgdr * kBoltzk;             // :126
constexpr double kRgas = (kRgasmol / kAmd) * 1000.0;       // :130
constexpr double kRwat = (kRgasmol / kAmw) * 1000.0;       // :131
constexpr double kCpd = 3.5 * kRgas;                       // :141
constexpr double kCvd = 2.5 * kRgas;                       // :145
constexpr double kWlhv = 2500610.0;                        // :167
constexpr double kRegrav = 1.0 / kEgrav;                   // :178
constexpr double kRcpd = 1.0 / kCpd;                       // :179
constexpr double kRovcp = kRgas * kRcpd;                   // :180
constexpr double kRdrcv = kRgas / kCvd;                    // :181
constexpr double kCpovr = kCpd / kRgas;                    // :182
constexpr double kTzero = 273.15;                          // :193
constexpr double kP00 = 1.000000e5;                        // :225
constexpr double kLrate = 0.00649;                         // :231
constexpr double kPi = 3.1415926535897932384626433832795029;  // :247
constexpr double kDegrad = kPi / 180.0;                    // :254
constexpr double kRaddeg = 180.0 / kPi;                    // :255
constexpr double kEarthrad = 6.371229e6;                   // :275
constexpr double kEomeg = 7.2921159e-5;                    // :279
constexpr double kEomeg2 = 2.0 * kEomeg;                   // :280
constexpr double kEp1 = kAmd / kAmw - 1.0;                 // :296
constexpr double kEp2 = kAmw / kAmd;                       // :299

// mod_moloch private parameters (nompi/mod_moloch.F90:95-106)
constexpr double kMinden = 1.0e-30;
constexpr double kXdamp = 0.0625;
constexpr double kNupaitq = 0.05;

// Flatau et al. (1992) 8th-order saturation-pressure polynomials
// (nompi/mod_moloch.F90:128-148), water (a) and ice (c) branches.
constexpr double kEsA0 = 0.611213476e+03;
constexpr double kEsA1 = 0.444007856e+02;
constexpr double kEsA2 = 0.143064234e+01;
constexpr double kEsA3 = 0.264461437e-01;
constexpr double kEsA4 = 0.305903558e-03;
constexpr double kEsA5 = 0.196237241e-05;
constexpr double kEsA6 = 0.892344772e-08;
constexpr double kEsA7 = -0.373208410e-10;
constexpr double kEsA8 = 0.209339997e-13;
constexpr double kEsC0 = 0.611123516e+03;
constexpr double kEsC1 = 0.503109514e+02;
constexpr double kEsC2 = 0.188369801e+01;
constexpr double kEsC3 = 0.420547422e-01;
constexpr double kEsC4 = 0.614396778e-03;
constexpr double kEsC5 = 0.602780717e-05;
constexpr double kEsC6 = 0.387940929e-07;
constexpr double kEsC7 = 0.149436277e-09;
constexpr double kEsC8 = 0.262655803e-12;

}  // namespace moloch
