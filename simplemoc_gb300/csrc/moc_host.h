// moc_host.h -- host helpers shared by the library's translation units.
#pragma once
#include <stdint.h>

#include "simplemoc_gb300.h"

// Checks sizes, index ranges and value domains of a host problem.
int moc_host_validate(const moc_dims *d, const moc_host *h);
// Builds the derived arrays the kernels read: 3D segment lengths per
// (2D track, polar, segment), cos(theta) per polar angle, the track weights,
// the sigma_t coefficient planes, and the transposed scatter table.
// *max_abs_dz = largest |ds * mu| (the height step of one segment).
// sigma_t coefficient planes [n_sigt][8][ldg] (see moc_internal.h).
void moc_host_coef(const moc_dims *d, const float *sigt, int32_t ldg, float *coef);
int moc_host_derive(const moc_dims *d, const moc_host *h, int32_t ldg, float *seg_ds, float *mu,
                    float *weight, float *coef, float *scatter_t, float *max_abs_dz);
