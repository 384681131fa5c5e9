// ref_shim.cpp -- C-linkage wrappers around the reference's own CPU kernels.
//
// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/liboracle_ref.so together
// with the reference's unmodified matlab/mex/src/*.cpp files (see Makefile);
// used by tests/ to pin the oracle restatement and to generate the committed
// fixtures in tests/golden/. The prototypes below are the reference's CPU
// kernel signatures (Ax_fan_mf.h:2-13, Atx_fan_mf.h:2-14, Ax_cone_mf.h:2-11,
// Atx_cone_mf.h:2-5); the reference compiles them with C++ linkage, which
// ctypes cannot call directly.

void Ax_fan_mf_cpu_siddon(float*, float*, float, float, float, int, int, int, float*, int, float*, int*);
void Ax_fan_mf_cpu_new(float*, float*, float, float, float, int, int, int, float*, int, float*, int*);
void Ax_fan_mf_cpu_new_fb(float*, float*, float, float, float, int, int, int, float*, int, float*, int*, float);
void Atx_fan_mf_cpu_new(float*, float*, float, float, float, int, int, float*, int, float*, float, float,
                        int, int*, int*, int, int, float*, float*, float*, float*);
void Atx_fan_mf_cpu_new_fb(float*, float*, float, float, float, int, int, float*, int, float*, float, int,
                           int*, int*, int, int, float*, float*, float*, float*);
void Ax_cone_mf_cpu_siddon(float*, float*, float, float, float, int, int, int, int, float*, float*, int, int,
                           float*, float*, int*, float);
void Ax_cone_mf_cpu_new(float*, float*, float*, float, float, float, int, int, int, int, float*, float*, int,
                        int, float*, float*, int*, float);
void Atx_cone_mf_cpu_new(float*, float*, float, float, float, int, int, int, float*, float*, float*, float,
                         float, float, float, int, int*, int*, int, int, float*, float*, int, int);

extern "C" {
void ref_Ax_fan_mf_cpu_siddon(float* X, float* y, float SO, float OD, float scale, int nx, int ny, int nv,
                              float* sd_phi, int nd, float* y_det, int* id_X)
{ Ax_fan_mf_cpu_siddon(X, y, SO, OD, scale, nx, ny, nv, sd_phi, nd, y_det, id_X); }

void ref_Ax_fan_mf_cpu_new(float* X, float* y, float SO, float OD, float scale, int nx, int ny, int nv,
                           float* sd_phi, int nd, float* y_det, int* id_X)
{ Ax_fan_mf_cpu_new(X, y, SO, OD, scale, nx, ny, nv, sd_phi, nd, y_det, id_X); }

void ref_Ax_fan_mf_cpu_new_fb(float* X, float* y, float SO, float OD, float scale, int nx, int ny, int nv,
                              float* sd_phi, int nd, float* y_det, int* id_X, float dy_det)
{ Ax_fan_mf_cpu_new_fb(X, y, SO, OD, scale, nx, ny, nv, sd_phi, nd, y_det, id_X, dy_det); }

void ref_Atx_fan_mf_cpu_new(float* x, float* Y, float SO, float OD, float scale, int nx, int ny, float* sd_phi,
                            int nd, float* y_det, float dy_det, float y_os, int nt, int* id_Y, int* Nv,
                            int tmp_size, int nv, float* cos_phi, float* sin_phi, float* cos_det, float* sin_det)
{ Atx_fan_mf_cpu_new(x, Y, SO, OD, scale, nx, ny, sd_phi, nd, y_det, dy_det, y_os, nt, id_Y, Nv, tmp_size, nv,
                     cos_phi, sin_phi, cos_det, sin_det); }

void ref_Atx_fan_mf_cpu_new_fb(float* x, float* Y, float SO, float OD, float scale, int nx, int ny,
                               float* sd_phi, int nd, float* y_det, float dy_det, int nt, int* id_Y, int* Nv,
                               int tmp_size, int nv, float* cos_phi, float* sin_phi, float* cos_det,
                               float* sin_det)
{ Atx_fan_mf_cpu_new_fb(x, Y, SO, OD, scale, nx, ny, sd_phi, nd, y_det, dy_det, nt, id_Y, Nv, tmp_size, nv,
                        cos_phi, sin_phi, cos_det, sin_det); }

void ref_Ax_cone_mf_cpu_siddon(float* X, float* y, float SO, float OD, float scale, int nx, int ny, int nz,
                               int nv, float* sd_phi, float* sd_z, int na, int nb, float* y_det, float* z_det,
                               int* id_X, float dz0)
{ Ax_cone_mf_cpu_siddon(X, y, SO, OD, scale, nx, ny, nz, nv, sd_phi, sd_z, na, nb, y_det, z_det, id_X, dz0); }

void ref_Ax_cone_mf_cpu_new(float* X, float* y, float* yNorm, float SO, float OD, float scale, int nx, int ny,
                            int nz, int nv, float* sd_phi, float* sd_z, int na, int nb, float* y_det,
                            float* z_det, int* id_X, float dz)
{ Ax_cone_mf_cpu_new(X, y, yNorm, SO, OD, scale, nx, ny, nz, nv, sd_phi, sd_z, na, nb, y_det, z_det, id_X, dz); }

void ref_Atx_cone_mf_cpu_new(float* x, float* Y, float SO, float OD, float scale, int nx, int ny, int nz,
                             float* sd_z, float* y_det, float* z_det, float dy_det, float y_os, float dz_det,
                             float dz, int nt, int* id_Y, int* Nv, int tmp_size, int nv, float* cos_phi,
                             float* sin_phi, int na, int nb)
{ Atx_cone_mf_cpu_new(x, Y, SO, OD, scale, nx, ny, nz, sd_z, y_det, z_det, dy_det, y_os, dz_det, dz, nt, id_Y,
                      Nv, tmp_size, nv, cos_phi, sin_phi, na, nb); }
}
