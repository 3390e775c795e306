// Declarations of the few BLAS entry points the reference's Matrix.cpp and
// friends call.  The oracle library links ref_blas.c, a plain column-major
// implementation, in place of Intel oneMKL.
#pragma once
enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
typedef enum CBLAS_LAYOUT CBLAS_ORDER;
typedef int MKL_INT;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
extern "C" {
void cblas_dgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, double,
                 const double*, int, const double*, int, double, double*, int);
void cblas_dgemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, int, int, double, const double*, int,
                 const double*, int, double, double*, int);
void cblas_sgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, float,
                 const float*, int, const float*, int, float, float*, int);
void cblas_sgemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, int, int, float, const float*, int,
                 const float*, int, float, float*, int);
void dgetrf(const int*, const int*, double*, const int*, int*, int*);
void dgetrs(const char*, const int*, const int*, const double*, const int*, const int*,
            double*, const int*, int*);
void dgbtrf(const int*, const int*, const int*, const int*, double*, const int*, int*, int*);
void dgbtrs(const char*, const int*, const int*, const int*, const int*, const double*,
            const int*, const int*, double*, const int*, int*);
void dsyev(const char*, const char*, const int*, double*, const int*, double*, double*,
           const int*, int*);
void dsyevr(const char*, const char*, const char*, const int*, double*, const int*,
            const double*, const double*, const int*, const int*, const double*, int*,
            double*, double*, const int*, int*, double*, const int*, int*, const int*, int*);
int LAPACKE_dsyevr(int, char, char, char, int, double*, int, double, double, int, int,
                   double, int*, double*, double*, int, int*);
int LAPACKE_dsyev(int, char, char, int, double*, int, double*);
void MKL_Set_Num_Threads(int);
void mkl_set_num_threads(int);
void pardisoinit(void*, const int*, int*);
void pardiso(void*, const int*, const int*, const int*, const int*, const int*,
             const void*, const int*, const int*, int*, const int*, int*, const int*,
             void*, void*, int*);
}
