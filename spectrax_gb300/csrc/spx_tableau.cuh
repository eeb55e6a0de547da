// spx_tableau.cuh — Prince & Dormand (1981) RK8(7)13M coefficients and the
// Diffrax-default step-size controller, shared by the single-solve and batched
// device steppers.
//
// Coefficients: P.J. Prince, J.R. Dormand, "High order embedded Runge-Kutta
// formulae", J. Comput. Appl. Math. 7(1), 1981 (the 8(7) pair Diffrax ships as
// Dopri8).  Each entry is the double nearest to the published rational; the
// error weights are the double differences b - bhat.
#pragma once
#include <cuda_runtime.h>

namespace spx {
namespace rk {

constexpr int S = 13;

__host__ __device__ constexpr double Cn(int i) {
  return i == 0 ? 0.0 : i == 1 ? 1.0 / 18.0 : i == 2 ? 1.0 / 12.0 : i == 3 ? 1.0 / 8.0
       : i == 4 ? 5.0 / 16.0 : i == 5 ? 3.0 / 8.0 : i == 6 ? 59.0 / 400.0 : i == 7 ? 93.0 / 200.0
       : i == 8 ? 5490023248.0 / 9719169821.0 : i == 9 ? 13.0 / 20.0
       : i == 10 ? 1201146811.0 / 1299019798.0 : 1.0;
}

// a(i, j), 0 <= j < i < 13 (0-based stages)
__host__ __device__ constexpr double A(int i, int j) {
  switch (i) {
    case 1: return j == 0 ? 1.0 / 18.0 : 0.0;
    case 2: return j == 0 ? 1.0 / 48.0 : j == 1 ? 1.0 / 16.0 : 0.0;
    case 3: return j == 0 ? 1.0 / 32.0 : j == 2 ? 3.0 / 32.0 : 0.0;
    case 4: return j == 0 ? 5.0 / 16.0 : j == 2 ? -75.0 / 64.0 : j == 3 ? 75.0 / 64.0 : 0.0;
    case 5: return j == 0 ? 3.0 / 80.0 : j == 3 ? 3.0 / 16.0 : j == 4 ? 3.0 / 20.0 : 0.0;
    case 6:
      return j == 0 ? 29443841.0 / 614563906.0 : j == 3 ? 77736538.0 / 692538347.0
           : j == 4 ? -28693883.0 / 1125000000.0 : j == 5 ? 23124283.0 / 1800000000.0 : 0.0;
    case 7:
      return j == 0 ? 16016141.0 / 946692911.0 : j == 3 ? 61564180.0 / 158732637.0
           : j == 4 ? 22789713.0 / 633445777.0 : j == 5 ? 545815736.0 / 2771057229.0
           : j == 6 ? -180193667.0 / 1043307555.0 : 0.0;
    case 8:
      return j == 0 ? 39632708.0 / 573591083.0 : j == 3 ? -433636366.0 / 683701615.0
           : j == 4 ? -421739975.0 / 2616292301.0 : j == 5 ? 100302831.0 / 723423059.0
           : j == 6 ? 790204164.0 / 839813087.0 : j == 7 ? 800635310.0 / 3783071287.0 : 0.0;
    case 9:
      return j == 0 ? 246121993.0 / 1340847787.0 : j == 3 ? -37695042795.0 / 15268766246.0
           : j == 4 ? -309121744.0 / 1061227803.0 : j == 5 ? -12992083.0 / 490766935.0
           : j == 6 ? 6005943493.0 / 2108947869.0 : j == 7 ? 393006217.0 / 1396673457.0
           : j == 8 ? 123872331.0 / 1001029789.0 : 0.0;
    case 10:
      return j == 0 ? -1028468189.0 / 846180014.0 : j == 3 ? 8478235783.0 / 508512852.0
           : j == 4 ? 1311729495.0 / 1432422823.0 : j == 5 ? -10304129995.0 / 1701304382.0
           : j == 6 ? -48777925059.0 / 3047939560.0 : j == 7 ? 15336726248.0 / 1032824649.0
           : j == 8 ? -45442868181.0 / 3398467696.0 : j == 9 ? 3065993473.0 / 597172653.0 : 0.0;
    case 11:
      return j == 0 ? 185892177.0 / 718116043.0 : j == 3 ? -3185094517.0 / 667107341.0
           : j == 4 ? -477755414.0 / 1098053517.0 : j == 5 ? -703635378.0 / 230739211.0
           : j == 6 ? 5731566787.0 / 1027545527.0 : j == 7 ? 5232866602.0 / 850066563.0
           : j == 8 ? -4093664535.0 / 808688257.0 : j == 9 ? 3962137247.0 / 1805957418.0
           : j == 10 ? 65686358.0 / 487910083.0 : 0.0;
    case 12:
      return j == 0 ? 403863854.0 / 491063109.0 : j == 3 ? -5068492393.0 / 434740067.0
           : j == 4 ? -411421997.0 / 543043805.0 : j == 5 ? 652783627.0 / 914296604.0
           : j == 6 ? 11173962825.0 / 925320556.0 : j == 7 ? -13158990841.0 / 6184727034.0
           : j == 8 ? 3936647629.0 / 1978049680.0 : j == 9 ? -160528059.0 / 685178525.0
           : j == 10 ? 248638103.0 / 1413531060.0 : 0.0;
    default: return 0.0;
  }
}

__host__ __device__ constexpr double B(int j) {
  return j == 0 ? 14005451.0 / 335480064.0 : j == 5 ? -59238493.0 / 1068277825.0
       : j == 6 ? 181606767.0 / 758867731.0 : j == 7 ? 561292985.0 / 797845732.0
       : j == 8 ? -1041891430.0 / 1371343529.0 : j == 9 ? 760417239.0 / 1151165299.0
       : j == 10 ? 118820643.0 / 751138087.0 : j == 11 ? -528747749.0 / 2220607170.0
       : j == 12 ? 1.0 / 4.0 : 0.0;
}

__host__ __device__ constexpr double Bhat(int j) {
  return j == 0 ? 13451932.0 / 455176623.0 : j == 5 ? -808719846.0 / 976000145.0
       : j == 6 ? 1757004468.0 / 5645159321.0 : j == 7 ? 656045339.0 / 265891186.0
       : j == 8 ? -3867574721.0 / 1518517206.0 : j == 9 ? 465885868.0 / 322736535.0
       : j == 10 ? 53011238.0 / 667516719.0 : j == 11 ? 2.0 / 45.0 : 0.0;
}

__host__ __device__ constexpr double E(int j) { return B(j) - Bhat(j); }

// Diffrax PIDController defaults: pcoeff=0, icoeff=1, dcoeff=0, safety 0.9,
// factormin 0.2, factormax 10, error order 8 (exponent -1/8).
constexpr double SAFETY = 0.9, FACTORMIN = 0.2, FACTORMAX = 10.0, EXPONENT = -1.0 / 8.0;
constexpr double SNAP = 1e-9;   // a step within SNAP*h of the next stop lands on it

__device__ __forceinline__ double controller_factor(double en, bool accepted) {
  double f;
  if (en == 0.0) f = FACTORMAX;
  else if (!isfinite(en)) f = FACTORMIN;
  else f = SAFETY * pow(en, EXPONENT);
  const double lo = accepted ? 1.0 : FACTORMIN;
  return fmin(fmax(f, lo), FACTORMAX);
}

}  // namespace rk
}  // namespace spx
