/*
 * CPU oracle for the FMM-KMC energy-difference path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C with OpenMP,
 * the arithmetic that ppmd/coulomb_kmc generates at runtime as C source.
 * It keeps the reference's data layout (halo-padded particle store
 * [lsd0,lsd1,lsd2,max_occ,5], local expansions [.., 2L^2] with the real
 * block first) and its loop structure, so that it serves both as the parity
 * checker of the GPU path and as the timed "restated reference CPU path".
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load
 * it; the product never does.
 *
 * Each function cites the reference file:line it follows (paths relative to
 * the coulomb_kmc project root).
 *
 * Spherical harmonics: the reference obtains them from ppmd's SphGen code
 * generator (not vendored).  Its own Python restatements
 * (coulomb_kmc/kmc_expansion_tools.py:384-491) pin the convention:
 *   Y_l^m = sqrt((l-|m|)!/(l+|m|)!) P_l^{|m|}(cos theta) e^{i m phi},
 * P with the Condon-Shortley phase (scipy lpmv).  Here P is produced by the
 * standard normalised three-term recurrence; tests check it against lpmv.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

typedef double REAL;
typedef int64_t INT64;

#define MAXL 32

/* cube index l(l+1)+m, kmc_expansion_tools.py:34 (cube_ind) */
#define CUBE_IND(l, m) ((l) * ((l) + 1) + (m))

/* spherical(): kmc_full_long_range.py:584-595 and common.py:6-34 */
static inline void spherical(REAL dx, REAL dy, REAL dz, REAL *radius, REAL *theta, REAL *phi)
{
    const REAL dx2 = dx * dx;
    const REAL dx2_p_dy2 = dx2 + dy * dy;
    const REAL d2 = dx2_p_dy2 + dz * dz;
    *radius = sqrt(d2);
    *theta = atan2(sqrt(dx2_p_dy2), dz);
    *phi = atan2(dy, dx);
}

/*
 * Y_l^m(theta, phi) for 0<=l<L, -l<=m<=l written at CUBE_IND(l, m).
 * Normalised associated Legendre recurrence:
 *   N_m^m     = -sqrt((2m-1)/(2m)) sin N_{m-1}^{m-1}
 *   N_{m+1}^m = sqrt(2m+1) cos N_m^m
 *   N_l^m     = ((2l-1) cos N_{l-1}^m - sqrt((l-1)^2-m^2) N_{l-2}^m) / sqrt(l^2-m^2)
 */
static void ylm_table(const int L, const REAL theta, const REAL phi, REAL *yre, REAL *yim)
{
    REAL N[MAXL][MAXL];
    const REAL ct = cos(theta);
    const REAL st = sqrt(1.0 - ct * ct); /* kmc_octal.py:606-607 */
    N[0][0] = 1.0;
    for (int m = 1; m < L; m++) N[m][m] = -sqrt((2.0 * m - 1.0) / (2.0 * m)) * st * N[m - 1][m - 1];
    for (int m = 0; m < L - 1; m++) N[m + 1][m] = sqrt(2.0 * m + 1.0) * ct * N[m][m];
    for (int m = 0; m < L; m++)
        for (int l = m + 2; l < L; l++)
            N[l][m] = ((2.0 * l - 1.0) * ct * N[l - 1][m] - sqrt((REAL)((l - 1) * (l - 1) - m * m)) * N[l - 2][m]) /
                      sqrt((REAL)(l * l - m * m));
    const REAL cp = cos(phi), sp = sin(phi);
    REAL cm = 1.0, sm = 0.0; /* cos(m phi), sin(m phi) by complex multiplication */
    for (int m = 0; m < L; m++) {
        for (int l = m; l < L; l++) {
            yre[CUBE_IND(l, m)] = N[l][m] * cm;
            yim[CUBE_IND(l, m)] = N[l][m] * sm;
            yre[CUBE_IND(l, -m)] = N[l][m] * cm;
            yim[CUBE_IND(l, -m)] = -N[l][m] * sm;
        }
        const REAL cn = cm * cp - sm * sp;
        const REAL sn = sm * cp + cm * sp;
        cm = cn;
        sm = sn;
    }
}

/* multipole_exp: out[re] += Re Y_l^{-m} q r^l ; out[im] += Im Y_l^{-m} q r^l
 * kmc_expansion_tools.py:38-100 */
void orc_multipole_exp(INT64 L, REAL charge, REAL radius, REAL theta, REAL phi, REAL *out)
{
    REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
    ylm_table((int)L, theta, phi, yre, yim);
    const INT64 IM = L * L;
    REAL rhol = 1.0;
    for (int l = 0; l < L; l++) {
        const REAL rc = rhol * charge;
        for (int m = -l; m <= l; m++) {
            out[CUBE_IND(l, m)] += yre[CUBE_IND(l, -m)] * rc;
            out[IM + CUBE_IND(l, m)] += yim[CUBE_IND(l, -m)] * rc;
        }
        rhol *= radius;
    }
}

/* local_dot_vec: out[re] += Re Y_l^m q r^l ; out[im] += -Im Y_l^m q r^l
 * kmc_expansion_tools.py:102-150 */
void orc_dot_vec(INT64 L, REAL charge, REAL radius, REAL theta, REAL phi, REAL *out)
{
    REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
    ylm_table((int)L, theta, phi, yre, yim);
    const INT64 IM = L * L;
    REAL rhol = 1.0;
    for (int l = 0; l < L; l++) {
        const REAL rc = rhol * charge;
        for (int m = -l; m <= l; m++) {
            out[CUBE_IND(l, m)] += yre[CUBE_IND(l, m)] * rc;
            out[IM + CUBE_IND(l, m)] += (-1.0) * yim[CUBE_IND(l, m)] * rc;
        }
        rhol *= radius;
    }
}

/* create_local_exp: out[re] += Re Y_l^{-m} q r^{-l-1} ; out[im] += Im Y_l^{-m} q r^{-l-1}
 * kmc_expansion_tools.py:177-262 */
void orc_local_exp(INT64 L, REAL charge, REAL radius, REAL theta, REAL phi, REAL *out)
{
    REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
    ylm_table((int)L, theta, phi, yre, yim);
    const INT64 IM = L * L;
    const REAL iradius = 1.0 / radius;
    REAL rhol = iradius;
    for (int l = 0; l < L; l++) {
        for (int m = -l; m <= l; m++) {
            out[CUBE_IND(l, m)] += yre[CUBE_IND(l, -m)] * rhol * charge;
            out[IM + CUBE_IND(l, m)] += yim[CUBE_IND(l, -m)] * rhol * charge;
        }
        rhol *= iradius;
    }
}

/* local_eval: sum_l r^l sum_m Re(L_lm Y_l^m)   kmc_expansion_tools.py:152-175 */
REAL orc_local_eval(INT64 L, REAL radius, REAL theta, REAL phi, const REAL *moments)
{
    REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
    ylm_table((int)L, theta, phi, yre, yim);
    const INT64 IM = L * L;
    REAL rhol = 1.0, e = 0.0;
    for (int l = 0; l < L; l++) {
        for (int m = -l; m <= l; m++) {
            const int i = CUBE_IND(l, m);
            e += rhol * (moments[i] * yre[i] - moments[IM + i] * yim[i]);
        }
        rhol *= radius;
    }
    return e;
}

/* ------------------------------------------------------------------------ */
/* move set-up: kmc_mpi_decomp.py:388-616 (single rank: local_offset = 0)   */
/* ------------------------------------------------------------------------ */

/* get_cell: kmc_mpi_decomp.py:400-430 */
static inline void get_cell(const REAL *position, const REAL *extent, const INT64 *ncps, const INT64 *upper_allowed,
                            const INT64 *lower_allowed, const INT64 periodic, INT64 *cell, REAL *shifted_position)
{
    REAL sp0 = position[0] + 0.5 * extent[0];
    REAL sp1 = position[1] + 0.5 * extent[1];
    REAL sp2 = position[2] + 0.5 * extent[2];
    const REAL w0 = ncps[0] / extent[0];
    const REAL w1 = ncps[1] / extent[1];
    const REAL w2 = ncps[2] / extent[2];
    cell[0] = (INT64)(sp0 * w0);
    cell[1] = (INT64)(sp1 * w1);
    cell[2] = (INT64)(sp2 * w2);
    if (cell[0] >= ncps[2]) cell[0] = ncps[2] - 1;
    if (cell[1] >= ncps[1]) cell[1] = ncps[1] - 1;
    if (cell[2] >= ncps[0]) cell[2] = ncps[0] - 1;
    if (!periodic) {
        shifted_position[0] = position[0];
        shifted_position[1] = position[1];
        shifted_position[2] = position[2];
    } else {
        /* kmc_mpi_decomp.py:368-385 */
        REAL off[3];
        off[0] = (cell[0] < lower_allowed[0]) ? 1.0 : 0.0;
        off[1] = (cell[1] < lower_allowed[1]) ? 1.0 : 0.0;
        off[2] = (cell[2] < lower_allowed[2]) ? 1.0 : 0.0;
        if (cell[0] > upper_allowed[0]) off[0] = -1.0;
        if (cell[1] > upper_allowed[1]) off[1] = -1.0;
        if (cell[2] > upper_allowed[2]) off[2] = -1.0;
        cell[0] += (INT64)off[0] * ncps[2];
        cell[1] += (INT64)off[1] * ncps[1];
        cell[2] += (INT64)off[2] * ncps[0];
        shifted_position[0] = position[0] + off[0] * extent[0];
        shifted_position[1] = position[1] + off[1] * extent[1];
        shifted_position[2] = position[2] + off[2] * extent[2];
    }
}

/* gcell_to_lcell: kmc_mpi_decomp.py:449-458 */
static inline INT64 gcell_to_lcell(const INT64 pad, const INT64 lsd, const INT64 *cell)
{
    return (cell[0] + pad) + lsd * ((cell[1] + pad) + lsd * (cell[2] + pad));
}

/* linear global cell -> xyz tuple: kmc_mpi_decomp.py:432-447 */
static inline void get_fmm_cell(const INT64 cc, const INT64 ncps, INT64 *cell)
{
    const INT64 cx = cc % ncps;
    const INT64 cycz = (cc - cx) / ncps;
    const INT64 cy = cycz % ncps;
    const INT64 cz = (cycz - cy) / ncps;
    cell[0] = cx;
    cell[1] = cy;
    cell[2] = cz;
}

/* Bin positions into linear global cells with get_cell (kmc_mpi_decomp.py:400-420). */
void orc_bin_cells(INT64 N, const REAL *positions, const REAL *extent, INT64 ncps_, INT64 *cells)
{
    const INT64 ncps[3] = {ncps_, ncps_, ncps_};
    const INT64 ua[3] = {ncps_ + 8, ncps_ + 8, ncps_ + 8}, la[3] = {-8, -8, -8};
    for (INT64 i = 0; i < N; i++) {
        INT64 c[3];
        REAL sp[3];
        get_cell(&positions[3 * i], extent, ncps, ua, la, 0, c, sp);
        cells[i] = c[0] + ncps_ * (c[1] + ncps_ * c[2]);
    }
}

/* check_move: kmc_mpi_decomp.py:460-486 */
static inline void check_move(const REAL *extent, const REAL *p, const REAL *pp, int *err, const INT64 periodic,
                              const REAL max_move_2)
{
    for (int d = 0; d < 3; d++) {
        if (pp[d] < -0.5 * extent[d]) err[0]++;
        if (pp[d] > 0.5 * extent[d]) err[0]++;
    }
    REAL dd[3] = {p[0] - pp[0], p[1] - pp[1], p[2] - pp[2]};
    if (periodic) {
        for (int d = 0; d < 3; d++) {
            if (dd[d] < (0.5 * extent[d])) dd[d] += extent[d];
            if (dd[d] > (0.5 * extent[d])) dd[d] -= extent[d];
        }
    }
    for (int d = 0; d < 3; d++)
        if ((dd[d] * dd[d]) > max_move_2) err[0]++;
}

/* setup_move: kmc_mpi_decomp.py:489-616 */
int orc_setup_move(const INT64 npart_local, const INT64 max_prop, const INT64 *site_max_counts,
                   const INT64 *current_sites, const REAL *current_positions, const REAL *current_charges,
                   const INT64 *current_ids, const INT64 *current_fmm_cells, const REAL *prop_positions,
                   const INT64 *prop_masks, const INT64 prop_charge_flag, const REAL *prop_charges,
                   INT64 *rate_location, REAL *new_positions, REAL *new_charges, INT64 *new_ids,
                   INT64 *new_fmm_cells, REAL *new_shifted_positions, REAL *old_positions, REAL *old_charges,
                   INT64 *old_ids, INT64 *old_fmm_cells, INT64 *exclusive_sum, INT64 *num_particles,
                   INT64 *total_movs, const REAL *extent, const INT64 ncps_, const INT64 pad, const INT64 lsd,
                   const INT64 periodic, const REAL max_move)
{
    const INT64 ncps[3] = {ncps_, ncps_, ncps_};
    /* single rank: cell indices run -pad .. ncps+pad-1; lower_allowed = cell_indices[1],
       upper_allowed = cell_indices[-2]  (kmc_mpi_decomp.py:86-90) */
    const INT64 la[3] = {-pad + 1, -pad + 1, -pad + 1};
    const INT64 ua[3] = {ncps_ + pad - 2, ncps_ + pad - 2, ncps_ + pad - 2};
    const REAL max_move_2 = max_move * max_move;
    int err = 0;
    INT64 es_tmp = 0, old_ind = 0;
    for (INT64 px = 0; px < npart_local; px++) {
        INT64 es_inner = 0, prop_found = 0;
        const INT64 max_prop_count = site_max_counts[current_sites[px]];
        for (INT64 movx = 0; (movx < max_prop) && (prop_found < max_prop_count); movx++) {
            if (prop_masks[px * max_prop + movx] > 0) {
                es_inner++;
                prop_found++;
            }
        }
        if (es_inner > 0) {
            exclusive_sum[old_ind] = es_tmp;
            es_tmp += es_inner;
            old_ids[old_ind] = px;
            old_ind++;
        }
    }
    exclusive_sum[old_ind] = es_tmp;
    *num_particles = old_ind;
    *total_movs = es_tmp;

#pragma omp parallel for schedule(dynamic) reduction(+ : err)
    for (INT64 oind = 0; oind < old_ind; oind++) {
        const INT64 px = old_ids[oind];
        for (int d = 0; d < 3; d++) old_positions[oind * 3 + d] = current_positions[px * 3 + d];
        old_charges[oind] = current_charges[px];
        old_ids[oind] = current_ids[px];
        INT64 tmp_cell[3];
        get_fmm_cell(current_fmm_cells[px], ncps_, tmp_cell);
        old_fmm_cells[oind] = gcell_to_lcell(pad, lsd, tmp_cell);
        const INT64 prop_count = exclusive_sum[oind + 1] - exclusive_sum[oind];
        const INT64 nstart = exclusive_sum[oind];
        INT64 prop_found = 0;
        for (INT64 movx = 0; (movx < max_prop) && (prop_found < prop_count); movx++) {
            if (prop_masks[px * max_prop + movx] > 0) {
                const INT64 nind = nstart + prop_found;
                const INT64 prop_ind = px * max_prop * 3 + movx * 3;
                for (int d = 0; d < 3; d++) new_positions[nind * 3 + d] = prop_positions[prop_ind + d];
                int e = 0;
                check_move(extent, &current_positions[px * 3], &prop_positions[prop_ind], &e, periodic, max_move_2);
                err += e;
                INT64 c[3];
                REAL sp[3];
                get_cell(&prop_positions[prop_ind], extent, ncps, ua, la, periodic, c, sp);
                new_fmm_cells[nind] = gcell_to_lcell(pad, lsd, c);
                for (int d = 0; d < 3; d++) new_shifted_positions[nind * 3 + d] = sp[d];
                new_charges[nind] = (prop_charge_flag > 0) ? prop_charges[px * max_prop + movx] : current_charges[px];
                new_ids[nind] = current_ids[px];
                rate_location[nind] = px * max_prop + movx;
                prop_found++;
            }
        }
    }
    return err;
}

/* ------------------------------------------------------------------------ */
/* near field: direct_new / direct_old  kmc_local.py:928-1031                */
/* ------------------------------------------------------------------------ */
int orc_direct(const INT64 exclude_self, const INT64 num_movs, const INT64 *offsets, const REAL *d_positions,
               const REAL *d_charges, const INT64 *d_ids, const INT64 *d_fmm_cells, const REAL *d_pdata,
               const INT64 *d_pdata_ids, const INT64 *d_cell_occ, const INT64 d_cell_stride, REAL *d_energy)
{
#pragma omp parallel for schedule(dynamic)
    for (INT64 idx = 0; idx < num_movs; idx++) {
        const INT64 ic = d_fmm_cells[idx];
        const REAL ipx = d_positions[idx * 3], ipy = d_positions[idx * 3 + 1], ipz = d_positions[idx * 3 + 2];
        REAL energy_red = 0.0;
        for (INT64 jcx = 0; jcx < 27; jcx++) {
            const INT64 jc = ic + offsets[jcx];
            const INT64 offset = jc * d_cell_stride;
            const INT64 offset5 = 5 * jc * d_cell_stride;
            for (INT64 jx = 0; jx < d_cell_occ[jc]; jx++) {
                const REAL dx = ipx - d_pdata[offset5 + jx * 5 + 0];
                const REAL dy = ipy - d_pdata[offset5 + jx * 5 + 1];
                const REAL dz = ipz - d_pdata[offset5 + jx * 5 + 2];
                const REAL jch = d_pdata[offset5 + jx * 5 + 3];
                const REAL r2 = dx * dx + dy * dy + dz * dz;
                const REAL contrib = jch / sqrt(r2);
                if (exclude_self)
                    energy_red += (d_pdata_ids[offset + jx] != d_ids[idx]) ? contrib : 0.0;
                else
                    energy_red += contrib;
            }
        }
        energy_red *= d_charges[idx];
        d_energy[idx] = energy_red;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* cell local expansion evaluation: indirect_interactions kmc_octal.py:569-707 */
/* ------------------------------------------------------------------------ */
int orc_indirect(const INT64 L, const INT64 num_movs, const INT64 *offsets, const REAL *d_centres,
                 const REAL *d_positions, const REAL *d_charges, const REAL *d_local_exp, REAL *d_energy)
{
    const INT64 ESTRIDE = 2 * L * L, HESTRIDE = L * L;
#pragma omp parallel for schedule(static)
    for (INT64 idx = 0; idx < num_movs; idx++) {
        const INT64 offset = offsets[idx];
        const REAL dx = d_positions[idx * 3 + 0] - d_centres[offset * 3 + 0];
        const REAL dy = d_positions[idx * 3 + 1] - d_centres[offset * 3 + 1];
        const REAL dz = d_positions[idx * 3 + 2] - d_centres[offset * 3 + 2];
        const REAL charge = d_charges[idx];
        const REAL *re_exp = &d_local_exp[ESTRIDE * offset];
        const REAL *im_exp = &d_local_exp[ESTRIDE * offset + HESTRIDE];
        const REAL radius = sqrt(dx * dx + dy * dy + dz * dz);
        const REAL phi = atan2(dy, dx);
        const REAL theta = atan2(sqrt(dx * dx + dy * dy), dz);
        REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
        ylm_table((int)L, theta, phi, yre, yim);
        REAL coeff = charge, e = 0.0;
        for (int l = 0; l < L; l++) {
            for (int m = -l; m <= l; m++) {
                const int i = CUBE_IND(l, m);
                e += coeff * (re_exp[i] * yre[i] - im_exp[i] * yim[i]);
            }
            coeff *= radius;
        }
        d_energy[idx] = e;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* self / moved-pair correction  kmc_fmm_self_interaction.py:48-55,149-267   */
/* ------------------------------------------------------------------------ */
static const int CELL_OFFSETS[27][3] = {
    {-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {-1, 1, -1}, {0, 1, -1}, {1, 1, -1},
    {-1, -1, 0},  {0, -1, 0},  {1, -1, 0},  {-1, 0, 0},  {0, 0, 0},  {1, 0, 0},  {-1, 1, 0},  {0, 1, 0},  {1, 1, 0},
    {-1, -1, 1},  {0, -1, 1},  {1, -1, 1},  {-1, 0, 1},  {0, 0, 1},  {1, 0, 1},  {-1, 1, 1},  {0, 1, 1},  {1, 1, 1},
}; /* common.py:53-81 */

int orc_self_interaction(const INT64 periodic27, const REAL *extent, const INT64 store_stride,
                         const INT64 num_particles, const INT64 *exclusive_sum, const REAL *old_positions,
                         const REAL *old_charges, const REAL *new_positions, REAL *out)
{
    REAL domain27 = 0.0; /* kmc_fmm_self_interaction.py:48-55 */
    for (int o = 0; o < 27; o++) {
        const REAL ox = extent[0] * CELL_OFFSETS[o][0], oy = extent[1] * CELL_OFFSETS[o][1],
                   oz = extent[2] * CELL_OFFSETS[o][2];
        if (CELL_OFFSETS[o][0] != 0 || CELL_OFFSETS[o][1] != 0 || CELL_OFFSETS[o][2] != 0)
            domain27 -= 1.0 / sqrt(ox * ox + oy * oy + oz * oz);
    }
#pragma omp parallel for schedule(dynamic)
    for (INT64 px = 0; px < num_particles; px++) {
        const REAL coeff = old_charges[px] * old_charges[px];
        const REAL opx = old_positions[3 * px], opy = old_positions[3 * px + 1], opz = old_positions[3 * px + 2];
        const INT64 nprop = exclusive_sum[px + 1] - exclusive_sum[px];
        for (INT64 movii = 0; movii < nprop; movii++) {
            const INT64 movi = movii + exclusive_sum[px];
            const REAL npx = new_positions[3 * movi], npy = new_positions[3 * movi + 1],
                       npz = new_positions[3 * movi + 2];
            const REAL dx = opx - npx, dy = opy - npy, dz = opz - npz;
            REAL energy27 = (1.0 / sqrt(dx * dx + dy * dy + dz * dz));
            if (periodic27) {
                energy27 = domain27;
                for (int o = 0; o < 27; o++) {
                    const REAL ddx = (extent[0] * CELL_OFFSETS[o][0] + opx) - npx;
                    const REAL ddy = (extent[1] * CELL_OFFSETS[o][1] + opy) - npy;
                    const REAL ddz = (extent[2] * CELL_OFFSETS[o][2] + opz) - npz;
                    energy27 += 1.0 / sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                }
            }
            out[store_stride * px + movii] = coeff * energy27;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* far-field lattice term  kmc_full_long_range.py:500-858                    */
/* ------------------------------------------------------------------------ */
/* apply_dipole_correction_split: kmc_full_long_range.py:521-540 */
static inline REAL dipole_split(const INT64 L, const REAL *dip, const REAL *M, const REAL *E)
{
    const INT64 H = L * L;
    const INT64 RE_1P1 = CUBE_IND(1, 1), RE_1_0 = CUBE_IND(1, 0), RE_1N1 = CUBE_IND(1, -1);
    REAL tmp = 0.0;
    tmp += (dip[0] * M[RE_1P1]) * E[RE_1P1];
    tmp += (dip[0] * M[RE_1P1]) * E[RE_1N1];
    tmp -= (dip[1] * M[H + RE_1P1]) * E[H + RE_1P1];
    tmp += (dip[1] * M[H + RE_1P1]) * E[H + RE_1N1];
    tmp += (dip[2] * M[RE_1_0]) * E[RE_1_0];
    return tmp;
}

/* linop_csr_both: kmc_full_long_range.py:609-633 */
static inline REAL linop_csr_both(const INT64 L, const REAL *data, const INT64 *indptr, const INT64 *indices,
                                  const REAL *x1, const REAL *E)
{
    const INT64 H = L * L;
    INT64 di = 0;
    REAL dot = 0.0;
    for (INT64 row = 0; row < H; row++) {
        REAL t1 = 0.0, t2 = 0.0;
        for (INT64 ci = indptr[row]; ci < indptr[row + 1]; ci++) {
            const INT64 col = indices[di];
            const REAL v = data[di];
            di++;
            t1 += v * x1[col];
            t2 += v * x1[col + H];
        }
        dot += t1 * E[row] + t2 * E[row + H];
    }
    return dot;
}

/* energy of a multipole / dot-vector pair: 0.5 * ((R M) . E + dip(M, E))
 * (kmc_full_long_range.py:116-118 via LongRangeMTL and dipole correction) */
REAL orc_lr_energy(const INT64 L, const REAL *data, const INT64 *indptr, const INT64 *indices, const REAL *dip,
                   const REAL *M, const REAL *E)
{
    return 0.5 * linop_csr_both(L, data, indptr, indices, M, E) + 0.5 * dipole_split(L, dip, M, E);
}

/* long_range_energy: kmc_full_long_range.py:710-858 (per-proposal copies of
 * M and E as in the reference, minus the OpenMP scratch management) */
int orc_long_range_energy(const INT64 L, const REAL old_energy, const INT64 store_stride, const INT64 num_particles,
                          const INT64 *exclusive_sum, const REAL *old_positions, const REAL *old_charges,
                          const REAL *new_positions, const REAL *new_charges, const REAL *existing_multipole,
                          const REAL *existing_evector, const REAL *data, const INT64 *indptr,
                          const INT64 *indices, const REAL *dip, REAL *out)
{
    const INT64 NC = 2 * L * L;
#pragma omp parallel for schedule(dynamic)
    for (INT64 px = 0; px < num_particles; px++) {
        REAL *old_moments = (REAL *)malloc(sizeof(REAL) * 4 * NC);
        REAL *old_evector = old_moments + NC;
        REAL *new_moments = old_evector + NC;
        REAL *new_evector = new_moments + NC;
        const REAL old_charge = old_charges[px];
        for (INT64 i = 0; i < NC; i++) {
            old_moments[i] = existing_multipole[i];
            old_evector[i] = existing_evector[i];
        }
        REAL r, t, p;
        spherical(old_positions[3 * px], old_positions[3 * px + 1], old_positions[3 * px + 2], &r, &t, &p);
        orc_multipole_exp(L, -1.0 * old_charge, r, t, p, old_moments);
        orc_dot_vec(L, -1.0 * old_charge, r, t, p, old_evector);
        const INT64 nprop = exclusive_sum[px + 1] - exclusive_sum[px];
        for (INT64 movii = 0; movii < nprop; movii++) {
            const INT64 movi = movii + exclusive_sum[px];
            for (INT64 i = 0; i < NC; i++) {
                new_moments[i] = old_moments[i];
                new_evector[i] = old_evector[i];
            }
            spherical(new_positions[3 * movi], new_positions[3 * movi + 1], new_positions[3 * movi + 2], &r, &t, &p);
            orc_multipole_exp(L, new_charges[movi], r, t, p, new_moments);
            orc_dot_vec(L, new_charges[movi], r, t, p, new_evector);
            const REAL new_energy = 0.5 * linop_csr_both(L, data, indptr, indices, new_moments, new_evector) +
                                    0.5 * dipole_split(L, dip, new_moments, new_evector);
            out[px * store_stride + movii] += old_energy - new_energy;
        }
        free(old_moments);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* energy difference assembly  kmc_fmm.py:583-663                            */
/* ------------------------------------------------------------------------ */
int orc_diff(const REAL energy_unit, const INT64 num_particles, const INT64 stride_si, const INT64 *exclusive_sum,
             const INT64 *rate_location, const REAL *U0D, const REAL *U0I, const REAL *U1D, const REAL *U1I,
             const REAL *USI, REAL *UDIFF)
{
#pragma omp parallel for schedule(dynamic)
    for (INT64 px = 0; px < num_particles; px++) {
        const INT64 es_start = exclusive_sum[px];
        const INT64 es_count = exclusive_sum[px + 1] - es_start;
        for (INT64 movx = 0; movx < es_count; movx++) {
            const INT64 u1loc = es_start + movx;
            UDIFF[rate_location[u1loc]] =
                (energy_unit) * (1.0 * (+U1D[u1loc] + U1I[u1loc] - U0D[px] - U0I[px]) - USI[px * stride_si + movx]);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* accept: incremental update of every stored cell's local expansion         */
/* accept_local_exp (INJECT_EXTRACT_FLAG == 0)  kmc_octal.py:961-1089        */
/* ------------------------------------------------------------------------ */
static inline int well_separated(INT64 t0, INT64 t1, INT64 t2, INT64 f0, INT64 f1, INT64 f2)
{
    return ((llabs(t0 - f0) < 2) && (llabs(t1 - f1) < 2) && (llabs(t2 - f2) < 2)) ? 0 : 1;
}

int orc_accept_local_exp(const INT64 L, const INT64 periodic27, const REAL *extent, const INT64 ncps,
                         const REAL charge, const REAL *new_pos, const REAL *old_pos, const INT64 *new_tuple,
                         const INT64 *old_tuple, const INT64 *cell_ind0, const INT64 *cell_ind1,
                         const INT64 *cell_ind2, const INT64 lsd0, const INT64 lsd1, const INT64 lsd2,
                         const REAL *orig_centres, REAL *local_expansions)
{
    const INT64 ESTRIDE = 2 * L * L;
    const int nimg = periodic27 ? 27 : 1;
#pragma omp parallel for schedule(dynamic) collapse(3)
    for (INT64 cz = 0; cz < lsd0; cz++)
        for (INT64 cy = 0; cy < lsd1; cy++)
            for (INT64 cx = 0; cx < lsd2; cx++) {
                REAL out[2 * MAXL * MAXL];
                REAL radius_vec[54], theta_vec[54], phi_vec[54], charge_vec[54];
                int bool_vec[54];
                const INT64 lin_cell = cx + lsd2 * (cy + lsd1 * cz);
                const REAL cxp = orig_centres[lin_cell * 3], cyp = orig_centres[lin_cell * 3 + 1],
                           czp = orig_centres[lin_cell * 3 + 2];
                const INT64 fx = cell_ind2[cx], fy = cell_ind1[cy], fz = cell_ind0[cz];
                REAL *cell_local_exp = &local_expansions[lin_cell * ESTRIDE];
                for (INT64 t = 0; t < ESTRIDE; t++) out[t] = 0.0;
                for (int pass = 0; pass < 2; pass++) {
                    const REAL *pos = pass == 0 ? old_pos : new_pos;
                    const INT64 *tup = pass == 0 ? old_tuple : new_tuple;
                    for (int ox = 0; ox < nimg; ox++) {
                        const INT64 o0 = periodic27 ? CELL_OFFSETS[ox][0] : 0;
                        const INT64 o1 = periodic27 ? CELL_OFFSETS[ox][1] : 0;
                        const INT64 o2 = periodic27 ? CELL_OFFSETS[ox][2] : 0;
                        /* kmc_octal.py:813-831: x takes the third offset component */
                        const REAL mpx = o2 * extent[0] + pos[0];
                        const REAL mpy = o1 * extent[1] + pos[1];
                        const REAL mpz = o0 * extent[2] + pos[2];
                        const INT64 mtx = o2 * ncps + tup[0];
                        const INT64 mty = o1 * ncps + tup[1];
                        const INT64 mtz = o0 * ncps + tup[2];
                        const int ws = well_separated(mtx, mty, mtz, fx, fy, fz);
                        const REAL dx = mpx - cxp, dy = mpy - cyp, dz = mpz - czp;
                        const REAL dx2_p_dy2 = dx * dx + dy * dy;
                        const REAL d2 = dx2_p_dy2 + dz * dz;
                        const int k = pass * nimg + ox;
                        radius_vec[k] = sqrt(d2);
                        theta_vec[k] = atan2(sqrt(dx2_p_dy2), dz);
                        phi_vec[k] = atan2(dy, dx);
                        charge_vec[k] = pass == 0 ? -1.0 * charge : charge;
                        bool_vec[k] = ws;
                    }
                }
                for (int k = 0; k < 2 * nimg; k++) {
                    const REAL iradius = bool_vec[k] ? 1.0 / radius_vec[k] : 0.0;
                    if (!bool_vec[k]) continue; /* contributions are exactly zero */
                    REAL yre[MAXL * MAXL], yim[MAXL * MAXL];
                    ylm_table((int)L, theta_vec[k], phi_vec[k], yre, yim);
                    REAL rhol = iradius * charge_vec[k];
                    for (int l = 0; l < L; l++) {
                        for (int m = -l; m <= l; m++) {
                            out[CUBE_IND(l, m)] += yre[CUBE_IND(l, -m)] * rhol;
                            out[L * L + CUBE_IND(l, m)] += yim[CUBE_IND(l, -m)] * rhol;
                        }
                        rhol *= iradius;
                    }
                }
                for (INT64 t = 0; t < ESTRIDE; t++) cell_local_exp[t] += out[t];
            }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* particle store update: extract + inject  kmc_local.py:180-371             */
/* old_locs / new_locs: per-dimension lists of store indices holding copies  */
/* ------------------------------------------------------------------------ */
int orc_store_extract(const INT64 gid, const INT64 n0, const INT64 *locs0, const INT64 n1, const INT64 *locs1,
                      const INT64 n2, const INT64 *locs2, const INT64 lsd, const INT64 max_occ, REAL *store,
                      INT64 *store_ids, INT64 *occ)
{
    if (n0 == 0 || n1 == 0 || n2 == 0) return 0;
    const INT64 c0 = locs0[0] + lsd * 0;
    const INT64 first = (locs0[0] * lsd + locs1[0]) * lsd + locs2[0];
    const INT64 old_occupancy = occ[first];
    INT64 index = -1, count = 0;
    for (INT64 j = 0; j < old_occupancy; j++)
        if (store_ids[first * max_occ + j] == gid) {
            index = j;
            count++;
        }
    (void)c0;
    if (count != 1) return -1; /* "Index was not unique" kmc_local.py:226-227 */
    for (INT64 a = 0; a < n0; a++)
        for (INT64 b = 0; b < n1; b++)
            for (INT64 c = 0; c < n2; c++) {
                const INT64 cell = (locs0[a] * lsd + locs1[b]) * lsd + locs2[c];
                occ[cell] = old_occupancy - 1;
                store_ids[cell * max_occ + index] = store_ids[cell * max_occ + old_occupancy - 1];
                for (int k = 0; k < 5; k++)
                    store[(cell * max_occ + index) * 5 + k] = store[(cell * max_occ + old_occupancy - 1) * 5 + k];
            }
    return 0;
}

int orc_store_inject(const INT64 gid, const REAL *new_position, const REAL charge, const INT64 n0,
                     const INT64 *locs0, const INT64 n1, const INT64 *locs1, const INT64 n2, const INT64 *locs2,
                     const REAL *pf0, const REAL *pf1, const REAL *pf2, const INT64 lsd, const INT64 max_occ,
                     const REAL *extent, const INT64 periodic, REAL *store, INT64 *store_ids, INT64 *occ)
{
    if (n0 == 0 || n1 == 0 || n2 == 0) return 0;
    const INT64 first = (locs0[0] * lsd + locs1[0]) * lsd + locs2[0];
    const INT64 old_occupancy = occ[first];
    if (old_occupancy + 1 > max_occ) return -2; /* caller resizes (kmc_local.py:314-316) */
    for (INT64 a = 0; a < n0; a++)
        for (INT64 b = 0; b < n1; b++)
            for (INT64 c = 0; c < n2; c++) {
                const INT64 cell = (locs0[a] * lsd + locs1[b]) * lsd + locs2[c];
                occ[cell] = old_occupancy + 1;
                store_ids[cell * max_occ + old_occupancy] = gid;
                REAL *s = &store[(cell * max_occ + old_occupancy) * 5];
                s[0] = new_position[0];
                s[1] = new_position[1];
                s[2] = new_position[2];
                s[3] = charge;
                memcpy(&s[4], &gid, sizeof(INT64));
                if (periodic) { /* kmc_local.py:345-357: slowest dim is z */
                    s[0] += pf2[c] * extent[0];
                    s[1] += pf1[b] * extent[1];
                    s[2] += pf0[a] * extent[2];
                }
            }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Initial finest-level local expansions (replaces ppmd PyFMM, which is not */
/* available): exact particle-to-local sum over every charge image that is   */
/* well separated from the cell, i.e. the state that accept_local_exp        */
/* maintains incrementally (kmc_octal.py:129-183).                           */
/* primary cells only, reference layout [ncps^3, 2L^2], cell = x fastest.    */
/* ------------------------------------------------------------------------ */
int orc_init_local_exp(const INT64 L, const INT64 periodic27, const REAL *extent, const INT64 ncps, const INT64 N,
                       const REAL *positions, const REAL *charges, const INT64 *fmm_cells, REAL *lexp)
{
    const INT64 NC = 2 * L * L;
    const INT64 ncell = ncps * ncps * ncps;
    const int nimg = periodic27 ? 27 : 1;
    const REAL w0 = extent[0] / ncps, w1 = extent[1] / ncps, w2 = extent[2] / ncps;
#pragma omp parallel for schedule(dynamic)
    for (INT64 c = 0; c < ncell; c++) {
        INT64 ct[3];
        get_fmm_cell(c, ncps, ct);
        /* cell centres: kmc_octal.py:397-428 (starts + cx * widths) */
        const REAL cxp = (-0.5 * extent[0] + 0.5 * w0) + ct[0] * w0;
        const REAL cyp = (-0.5 * extent[1] + 0.5 * w1) + ct[1] * w1;
        const REAL czp = (-0.5 * extent[2] + 0.5 * w2) + ct[2] * w2;
        REAL *out = &lexp[c * NC];
        for (INT64 t = 0; t < NC; t++) out[t] = 0.0;
        for (INT64 j = 0; j < N; j++) {
            INT64 jt[3];
            get_fmm_cell(fmm_cells[j], ncps, jt);
            for (int ox = 0; ox < nimg; ox++) {
                const INT64 o0 = periodic27 ? CELL_OFFSETS[ox][0] : 0;
                const INT64 o1 = periodic27 ? CELL_OFFSETS[ox][1] : 0;
                const INT64 o2 = periodic27 ? CELL_OFFSETS[ox][2] : 0;
                if (!well_separated(o2 * ncps + jt[0], o1 * ncps + jt[1], o0 * ncps + jt[2], ct[0], ct[1], ct[2]))
                    continue;
                const REAL dx = (o2 * extent[0] + positions[3 * j]) - cxp;
                const REAL dy = (o1 * extent[1] + positions[3 * j + 1]) - cyp;
                const REAL dz = (o0 * extent[2] + positions[3 * j + 2]) - czp;
                REAL r, t, p;
                spherical(dx, dy, dz, &r, &t, &p);
                orc_local_exp(L, charges[j], r, t, p, out);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Direct-sum oracles restated from the reference's tests                    */
/* FreeSpaceDirect: tests/host/test_common.py:24-55                          */
/* NearestDirect:   tests/host/test_common.py:61-103                         */
/* ------------------------------------------------------------------------ */
REAL orc_direct_energy(const INT64 periodic27, const REAL E, const INT64 N, const REAL *P, const REAL *Q)
{
    REAL phi = 0.0;
#pragma omp parallel for schedule(dynamic) reduction(+ : phi)
    for (INT64 i = 0; i < N; i++) {
        REAL inner = 0.0;
        for (INT64 j = i + 1; j < N; j++) {
            const REAL dx = P[3 * i] - P[3 * j], dy = P[3 * i + 1] - P[3 * j + 1], dz = P[3 * i + 2] - P[3 * j + 2];
            inner += Q[i] * Q[j] / sqrt(dx * dx + dy * dy + dz * dz);
        }
        if (periodic27) {
            for (INT64 j = 0; j < N; j++)
                for (int a = -1; a <= 1; a++)
                    for (int b = -1; b <= 1; b++)
                        for (int c = -1; c <= 1; c++) {
                            if (a == 0 && b == 0 && c == 0) continue;
                            const REAL dx = P[3 * j] - P[3 * i] + a * E;
                            const REAL dy = P[3 * j + 1] - P[3 * i + 1] + b * E;
                            const REAL dz = P[3 * j + 2] - P[3 * i + 2] + c * E;
                            inner += 0.5 * Q[i] * Q[j] / sqrt(dx * dx + dy * dy + dz * dz);
                        }
        }
        phi += inner;
    }
    return phi;
}
