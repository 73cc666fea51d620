// Solid-harmonic recurrences shared by the propose, accept and initial-solve
// kernels.
//
// Convention (the reference's, coulomb_kmc/kmc_expansion_tools.py:384-491):
//   Y_l^m = sqrt((l-|m|)!/(l+|m|)!) P_l^{|m|}(cos theta) e^{i m phi}, with the
//   Condon-Shortley phase.  Local expansions are stored for m >= 0 only
//   ("folded": L_{l,-m} = conj(L_{l,m}) holds for expansions of real charges),
//   at index h(l,m) = l(l+1)/2 + m.
//
// Instead of the reference's atan2/cos/sin route, harmonics are generated as
// Cartesian solid harmonics, which needs no trigonometry:
//   regular   Rg_l^m(x) = r^l      N_l^m P_l^m(cos) e^{+i m phi}
//   irregular Ir_l^m(x) = r^{-l-1} N_l^m P_l^m(cos) e^{-i m phi}
//   Rg_m^m = d_m (x + i y) Rg_{m-1}^{m-1},   Ir_m^m = d_m (x - i y)/r^2 Ir_{m-1}^{m-1}
//   Rg_l^m = a_lm z Rg_{l-1}^m - b_lm r^2 Rg_{l-2}^m
//   Ir_l^m = a_lm z/r^2 Ir_{l-1}^m - b_lm /r^2 Ir_{l-2}^m
// with a_lm = (2l-1)/sqrt(l^2-m^2), b_lm = sqrt((l-1)^2-m^2)/sqrt(l^2-m^2),
// d_m = -sqrt((2m-1)/(2m)).
//   local evaluation   phi(x) = sum Re(L_lm Rg_l^m(x))        (kmc_octal.py:569-707)
//   particle-to-local  L_lm  += q Ir_l^m(s)                     (kmc_expansion_tools.py:177-262)
//   multipole          M_lm  += q conj(Rg_l^m(s))               (kmc_expansion_tools.py:38-100)
#pragma once

#define KMC_LMAX 32

// recurrence coefficients, index l * KMC_LMAX + m
__constant__ double c_rec_a[KMC_LMAX * KMC_LMAX];
__constant__ double c_rec_b[KMC_LMAX * KMC_LMAX];
__constant__ double c_rec_d[KMC_LMAX];
// the same coefficients as FP32 pairs (hi, lo) for double-FP32 arithmetic
__constant__ float2 c_rec_a2[KMC_LMAX * KMC_LMAX];
__constant__ float2 c_rec_b2[KMC_LMAX * KMC_LMAX];
__constant__ float2 c_rec_d2[KMC_LMAX];

// Scaled particle-to-local recurrence (accept path): with J_l^m = Ir_l^m / C_lm,
//   C_mm = prod_{k<=m} d_k,  C_lm = a_lm C_{l-1,m},
//   J_m^m = q r^{-1} ((x - i y)/r^2)^m,  J_l^m = (z/r^2) J_{l-1}^m - beta_lm r^{-2} J_{l-2}^m,
//   beta_lm = b_lm / (a_lm a_{l-1,m})
// so the recurrence needs one coefficient product per step; C_lm is applied once
// per output in FP64.
__constant__ float2 c_p2l_beta[KMC_LMAX * KMC_LMAX];
__constant__ double c_p2l_scale[KMC_LMAX * KMC_LMAX];

__host__ __device__ inline int hidx(int l, int m) { return (l * (l + 1)) / 2 + m; }

// phi(x) = sum_{l<L} sum_{|m|<=l} Re(L_lm Rg_l^m(x)) for a folded expansion.
__device__ __forceinline__ double far_eval_fp64(const double2 *__restrict__ Lc, const int L, const double x,
                                                const double y, const double z)
{
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0;
    double total = 0.0;
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const double t = c_rec_d[m];
            const double nre = t * (dre * x - dim * y);
            const double nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        double2 Lv = __ldg(&Lc[hidx(m, m)]);
        double acc = Lv.x * cre - Lv.y * cim;
        for (int l = m + 1; l < L; ++l) {
            const double az = c_rec_a[l * KMC_LMAX + m] * z;
            const double br = c_rec_b[l * KMC_LMAX + m] * r2;
            const double nre = az * cre - br * pre;
            const double nim = az * cim - br * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            Lv = __ldg(&Lc[hidx(l, m)]);
            acc += Lv.x * cre - Lv.y * cim;
        }
        total += (m == 0) ? acc : 2.0 * acc;
    }
    return total;
}

// out[h(l,m)] = q conj(Rg_l^m(x)) for m >= 0 (a charge's multipole about the origin).
__device__ __forceinline__ void multipole_fp64(double2 *out, const int L, const double q, const double x,
                                               const double y, const double z)
{
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0;
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const double t = c_rec_d[m];
            const double nre = t * (dre * x - dim * y);
            const double nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        out[hidx(m, m)] = make_double2(q * cre, -q * cim);
        for (int l = m + 1; l < L; ++l) {
            const double az = c_rec_a[l * KMC_LMAX + m] * z;
            const double br = c_rec_b[l * KMC_LMAX + m] * r2;
            const double nre = az * cre - br * pre;
            const double nim = az * cim - br * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            out[hidx(l, m)] = make_double2(q * cre, -q * cim);
        }
    }
}
