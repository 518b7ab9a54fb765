// kernels.h -- host-side launchers of the atmosphere LUT build kernels.
#pragma once

#include <cuda_runtime.h>

#include "atmo_params.h"

namespace sfsim {

template <class Real>
struct SetupBuffers {
  Remap4<Real>* remapS;
  CellGeom<Real>* geom;
  Remap2<Real>* remapT;
  Remap2<Real>* remapE;
  RowInfo* rowinfo;
  RowSample<Real>* rows;
  SphereDir<Real>* sdirs;
};

template <class Real>
void launch_setup(const AtmoParams* params, const BuildDims& d, const DirLocal* dirs, const int* ring_end,
                  const SetupBuffers<Real>& o, cudaStream_t st);

template <class Real>
void launch_transmittance(const AtmoParams* params, const BuildDims& d, Vec4<Real>* T, cudaStream_t st);

template <class Real>
void launch_surface_base(const AtmoParams* params, const BuildDims& d, Vec4<Real>* E0, cudaStream_t st);

// First-order Rayleigh ray scatter and Mie strength (fused).
template <class Real>
void launch_first_order(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                        const RowSample<Real>* rows, const CellGeom<Real>* geom, Vec4<Real>* rayleigh,
                        Vec4<Real>* mie, cudaStream_t st);

template <class Real>
void launch_first_order_census(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                               const RowSample<Real>* rows, const CellGeom<Real>* geom, unsigned long long* count,
                               cudaStream_t st);

// Throughput probe of the SFU: `iters` ex2.approx per chain, 8 chains per thread.
void launch_sfu_probe(int blocks, int threads, int iters, float* sink, cudaStream_t st);

// J = point scatter of (dS, dE); when `mie` is non-NULL dS is the first
// iteration's rayleigh + mie * phase(mie, v.l).
template <class Real>
int launch_point_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                         const SphereDir<Real>* sdirs, const CellGeom<Real>* geom, const Vec4<Real>* dS,
                         const Vec4<Real>* mie, const Vec4<Real>* dE, Vec4<Real>* J, cudaStream_t st);

// dE = surface radiance of dS (same first-iteration convention).
template <class Real>
void launch_surface_radiance(const AtmoParams* params, const BuildDims& d, const DirLocal* half_dirs,
                             const Vec4<Real>* dS, const Vec4<Real>* mie, Vec4<Real>* dE, cudaStream_t st);

// dS = ray scatter of J.
template <class Real>
int launch_ray_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const Remap4<Real>* remap,
                       const Vec4<Real>* J, Vec4<Real>* dS, cudaStream_t st);

// out = re-interpolation of (a + b) at the node maps; b may be NULL and, for
// the 2-D variant, a may be NULL.
template <class Real>
void launch_accumulate4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st);

template <class Real>
void launch_accumulate2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st);

// Final tables in the .scatter layout (float RGB, 4-D tables tiled 2-D).
template <class Real>
void launch_output4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st);

template <class Real>
void launch_output2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st);

// Plain-order float copy of an internal table (debug intermediates).
template <class Real>
void launch_export(long long n, const Vec4<Real>* tab, float* out, cudaStream_t st);

}  // namespace sfsim
