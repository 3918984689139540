// Cartesian Gaussian shells: the components x^i y^j z^k of a shell of angular
// momentum l (l <= 2) in pyscf's Cartesian order (i = l..0, then j = l-i..0,
// k = l-i-j): s; x, y, z; xx, xy, xz, yy, yz, zz.  Each component is the
// monomial times the shell's radial sum c_p exp(-a_p r^2) (coefficients carry
// the normalisation), as pyscf's GTOval_cart / int*_cart give it.
#pragma once

constexpr int kMaxShellL = 2;

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// exponents (i, j, k) of component k of a shell of angular momentum l
__device__ inline void cart_exponents(int l, int k, int* c) {
  int i = l;
  for (; i > 0; --i) {
    const int cnt = l - i + 1;
    if (k < cnt) break;
    k -= cnt;
  }
  c[0] = i;
  c[1] = l - i - k;
  c[2] = k;
}

// d^e for e <= 2
__device__ inline double cart_pow(double d, int e) { return e == 0 ? 1.0 : (e == 1 ? d : d * d); }

// d/dd of d^e, e <= 2
__device__ inline double cart_dpow(double d, int e) { return e == 0 ? 0.0 : (e == 1 ? 1.0 : 2.0 * d); }
