// Test infrastructure: C entry point around the reference's own trk2dictionary
// (commit/trk2dictionary/trk2dictionary_c.cpp:111-287, compiled from the reference's
// source by oracle/build_ref.py into oracle/_ref), so the tests can run the reference's
// voxelisation on a .trk file and read back its dictionary_*.dict files.
#include <sys/stat.h>

#include <string>

int trk2dictionary(char *str_filename, int data_offset, int Nx, int Ny, int Nz, float Px, float Py, float Pz,
                   int n_count, int n_scalars, int n_properties, float fiber_shiftX, float fiber_shiftY,
                   float fiber_shiftZ, float min_seg_len, float min_fiber_len, float max_fiber_len, float *ptrPEAKS,
                   int Np, float vf_THR, int ECix, int ECiy, int ECiz, float *_ptrMASK, float *_ptrISO,
                   double **ptrTDI, char *path_out, int c, double *ptrPeaksAffine, int nReplicas,
                   double *ptrBlurRho, double *ptrBlurAngle, double *ptrBlurWeights, bool *ptrBlurApplyTo,
                   float *ptrToVOXMM, short *ptrHashTable, int threads_count, int verbose);

// out_dir receives the EC / ISO files, out_dir/temp the IC / TRK files of the single thread
// (index 0); tdi: Nx*Ny*Nz doubles (C order over x, y, z)
extern "C" int t2d_ref_run(const char *trk_path, int n_count, int Nx, int Ny, int Nz, float Px, float Py, float Pz,
                           float shift_x, float shift_y, float shift_z, float min_seg_len, float min_fiber_len,
                           float max_fiber_len, int do_intersect, float *mask, float *iso_mask, float *peaks, int Np,
                           float vf_thr, double *peaks_affine, int n_rep, double *rho, double *angle, double *w,
                           unsigned char *blur_apply, short *hash, double *tdi, const char *out_dir) {
    std::string out(out_dir);
    std::string tmp = out + "/temp";
    mkdir(out.c_str(), 0755);
    mkdir(tmp.c_str(), 0755);
    bool *ba = new bool[n_count > 0 ? n_count : 1];
    for (int i = 0; i < n_count; ++i) ba[i] = blur_apply ? blur_apply[i] != 0 : false;
    float to_voxmm[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    double *tdis[1] = {tdi};
    const int rc = trk2dictionary((char *)trk_path, 1000, Nx, Ny, Nz, Px, Py, Pz, n_count, 0, 0, shift_x, shift_y,
                                  shift_z, min_seg_len, min_fiber_len, max_fiber_len, peaks, Np, vf_thr, 1, 1, 1, mask,
                                  iso_mask, tdis, (char *)tmp.c_str(), do_intersect, peaks_affine, n_rep, rho, angle, w,
                                  ba, to_voxmm, hash, 1, 0);
    delete[] ba;
    return rc;
}
