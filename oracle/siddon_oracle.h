/* ORACLE -- test infrastructure only.  C interface of oracle/siddon_oracle.c. */
#ifndef SIDDON_ORACLE_H
#define SIDDON_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_OK = 0, ORACLE_EINVAL = 1 };
enum { ORACLE_PJ = 0, ORACLE_BPJ = 1, ORACLE_PJT = 2, ORACLE_BPJT = 3 };
enum { ORACLE_NONE = 0, ORACLE_SUN = 1 };

/* Cube header: CDELT1-3, PSHAPE1-3, MMIN1-3, MMAX1-3 (map_header). */
typedef struct {
  double cdelt[3], pshape[3], mmin[3], mmax[3];
} oracle_map_header;

/* View header: CRPIX1-2, CDELT1-2, CRVAL1-2, M1-3, R1_1..R3_3 row-major (image_header). */
typedef struct {
  double crpix[2], cdelt[2], crval[2], M[3], R[9];
} oracle_image_header;

int oracle_conic_full_projector_f64(const oracle_map_header *mh, const oracle_image_header *views, int T,
                                    double *data, long long n1, long long n2, const long long ds[3],
                                    double *map, const long long mshape[3], const long long ms[4],
                                    const double *mask, const long long ks[3],
                                    int obstacle, int mode, int nthread);
int oracle_conic_full_projector_f32(const oracle_map_header *mh, const oracle_image_header *views, int T,
                                    float *data, long long n1, long long n2, const long long ds[3],
                                    float *map, const long long mshape[3], const long long ms[4],
                                    const float *mask, const long long ks[3],
                                    int obstacle, int mode, int nthread);
int oracle_full_unit_vector_f64(const oracle_image_header *views, int T, const double *data,
                                long long n1, long long n2, const long long ds[3],
                                double *u, const long long us[4]);
int oracle_full_intersection_parameters_f64(const oracle_map_header *mh, const oracle_image_header *views,
                                            int T, long long n1, long long n2, const double *u,
                                            const long long us[4], double *a1, double *an);
int oracle_version(void);

#ifdef __cplusplus
}
#endif
#endif
