// moc_host.h -- host helpers shared by the library's translation units.
#pragma once
#include <stdint.h>

#include "simplemoc_gb300.h"

// Checks sizes, index ranges and value domains of a host problem.
int moc_host_validate(const moc_dims *d, const moc_host *h);
// The same checks in two parts: all but the per-segment source ids, and the
// source ids k in [first, end) of seg_src.
int moc_host_validate_except_ids(const moc_dims *d, const moc_host *h);
int moc_host_validate_ids(const moc_dims *d, const int32_t *seg_src, int64_t first, int64_t end);
// Builds the derived arrays the kernels read: 3D segment lengths per
// (2D track, polar, segment), cos(theta) per polar angle, the track weights,
// the sigma_t coefficient planes, and the transposed scatter table.
// *max_abs_dz = largest |ds * mu| (the height step of one segment).
// sigma_t coefficient planes [n_sigt][8][ldg] (see moc_internal.h).
// Coefficients of each sigma_t row, interleaved per 4-group chunk so that the
// planes of one chunk are 96 contiguous bytes (one base pointer, immediate
// offsets): coef[(row * ldg / 4 + c) * 24 + plane * 4 + e] for group 4c + e,
//   plane 0 sigT      1 1/sigT     2 1/sigT^2     3 1/(sigT sigT^2)
//         4 1/((3 sigT^2) sigT^2)  5 2/(sigT sigT^2)
// The divisors are the reference's float products (src/solver.c:153,176,198)
// and planes 1-4 their correctly rounded float reciprocals, with which PLAIN
// divides exactly; plane 5 is exactly twice plane 3 (MIXED).  A row takes
// MOC_COEF_PLANES * ldg floats.
enum { MOC_COEF_PLANES = 6 };
void moc_host_coef(const moc_dims *d, const float *sigt, int32_t ldg, float *coef);
int moc_host_derive(const moc_dims *d, const moc_host *h, int32_t ldg, float *seg_ds, float *mu,
                    float *weight, float *coef, float *scatter_t, float *max_abs_dz);
