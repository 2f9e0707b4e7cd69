// Project-written stand-in for libvvhd/src/TMatrix.cpp, whose solver calls LAPACK/CBLAS
// (absent here). TEST INFRASTRUCTURE ONLY.
//
// Keeps the class's bookkeeping semantics (solution pointer map, bodyMatrixIsOk flag,
// cached factorisation reused while the matrix bytes are unchanged) so calc_circulation
// takes the same fill paths as with LAPACK. The solve itself is a partial-pivot LU written
// here; it agrees with dgesv/dgetri+dgemv to rounding. The last filled system is recorded
// for the harness to export.
#include "TMatrix.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

std::vector<double> vvr_last_matrix, vvr_last_rhs, vvr_last_solution;

Matrix::Matrix()
    : N(0), BodyMatrix(), InverseMatrix(), RightCol(), ipvt(), solution_idx(), solution_ptr(),
      bodyMatrixHash_(), bodyMatrixIsOk_() {}

Matrix::~Matrix() {
    free(BodyMatrix);
    free(InverseMatrix);
    free(RightCol);
    free(ipvt);
}

void Matrix::resize(unsigned newsize) {
    if (newsize == N) return;
    N = newsize;
    BodyMatrix = (double*)realloc(BodyMatrix, N * N * sizeof(double));
    InverseMatrix = (double*)realloc(InverseMatrix, N * N * sizeof(double));
    RightCol = (double*)realloc(RightCol, N * sizeof(double));
    ipvt = (int*)realloc(ipvt, (N + 1) * sizeof(int));
    solution_ptr.resize(N);
    bodyMatrixIsOk_ = false;
}

double* Matrix::getCell(unsigned row, const double* solution) {
    unsigned col = getColForSolution(solution);
    if (row >= N || col >= N) {
        fprintf(stderr, "matrix shim: getCell(%u, %u) beyond limit\n", row, col);
        abort();
    }
    return BodyMatrix + (size_t)row * N + col;
}

double* Matrix::getRightCol(unsigned eq) {
    if (eq >= N) {
        fprintf(stderr, "matrix shim: getRightCol(%u) beyond limit\n", eq);
        abort();
    }
    return RightCol + eq;
}

void Matrix::setSolutionForCol(unsigned col, double* ptr) {
    solution_idx.erase(solution_ptr[col]);
    solution_ptr[col] = ptr;
    solution_idx[ptr] = col;
}

double* Matrix::getSolutionForCol(unsigned col) { return solution_ptr.at(col); }

unsigned Matrix::getColForSolution(const double* ptr) {
    auto it = solution_idx.find(ptr);
    return it != solution_idx.end() ? it->second : (unsigned)-1;
}

void Matrix::selfTest() {}

uint32_t Matrix::SuperFastHash(const char* data, int len) {
    // FNV-1a; only used to detect an unchanged matrix.
    uint32_t h = 2166136261u;
    for (int i = 0; i < len; i++) { h ^= (uint8_t)data[i]; h *= 16777619u; }
    return h;
}

static int shim_lu(size_t n, double* A, int* piv) {
    for (size_t k = 0; k < n; k++) {
        size_t p = k;
        double best = std::fabs(A[k * n + k]);
        for (size_t i = k + 1; i < n; i++) {
            double v = std::fabs(A[i * n + k]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = (int)p;
        if (best == 0) return -1;
        if (p != k)
            for (size_t j = 0; j < n; j++) std::swap(A[k * n + j], A[p * n + j]);
        double d = A[k * n + k];
        for (size_t i = k + 1; i < n; i++) {
            double l = A[i * n + k] / d;
            A[i * n + k] = l;
            if (l == 0) continue;
            for (size_t j = k + 1; j < n; j++) A[i * n + j] -= l * A[k * n + j];
        }
    }
    return 0;
}

static void shim_lu_solve(size_t n, const double* LU, const int* piv, double* b) {
    // rows were swapped whole during factorisation: permute b first, then forward-solve
    for (size_t k = 0; k < n; k++)
        if ((size_t)piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (size_t k = 0; k < n; k++)
        for (size_t i = k + 1; i < n; i++) b[i] -= LU[i * n + k] * b[k];
    for (size_t k = n; k-- > 0;) {
        double s = b[k];
        for (size_t j = k + 1; j < n; j++) s -= LU[k * n + j] * b[j];
        b[k] = s / LU[k * n + k];
    }
}

void Matrix::FillInverseMatrix() {
    // Here "InverseMatrix" holds the LU factors, reused while the matrix is unchanged.
    if (!bodyMatrixIsOk_) {
        fprintf(stderr, "matrix shim: cannot factorise without bodyMatrix\n");
        abort();
    }
    uint32_t hash = SuperFastHash((char*)BodyMatrix, (int)(N * N * sizeof(double)));
    if (hash == bodyMatrixHash_) return;
    memcpy(InverseMatrix, BodyMatrix, N * N * sizeof(double));
    if (shim_lu(N, InverseMatrix, ipvt)) {
        fprintf(stderr, "matrix shim: singular matrix\n");
        abort();
    }
    bodyMatrixHash_ = hash;
    bodyMatrixIsOk_ = false;
}

void Matrix::solveUsingInverseMatrix(bool useInverseMatrix) {
    vvr_last_matrix.assign(BodyMatrix, BodyMatrix + N * N);
    vvr_last_rhs.assign(RightCol, RightCol + N);
    std::vector<double> x(RightCol, RightCol + N);
    if (useInverseMatrix) {
        FillInverseMatrix();
        shim_lu_solve(N, InverseMatrix, ipvt, x.data());
    } else {
        if (!bodyMatrixIsOk_) {
            fprintf(stderr, "matrix shim: cannot solve SLAE without bodyMatrix\n");
            abort();
        }
        std::vector<double> A(BodyMatrix, BodyMatrix + N * N);
        std::vector<int> piv(N + 1);
        if (shim_lu(N, A.data(), piv.data())) {
            fprintf(stderr, "matrix shim: singular matrix\n");
            abort();
        }
        shim_lu_solve(N, A.data(), piv.data(), x.data());
        bodyMatrixIsOk_ = false;
    }
    for (size_t i = 0; i < N; i++) *solution_ptr[i] = x[i];
    vvr_last_solution = x;
}

void Matrix::transpose(double* A, unsigned n) {
    for (unsigned i = 0; i < n; i++)
        for (unsigned j = i + 1; j < n; j++) std::swap(A[i * n + j], A[j * n + i]);
}

void Matrix::save(const char*) {}

void Matrix::fillWithZeros() {
    bodyMatrixIsOk_ = false;
    memset(BodyMatrix, 0, N * N * sizeof(double));
    memset(RightCol, 0, N * sizeof(double));
}

bool Matrix::testNan() {
    for (size_t i = 0; i < N * N; i++)
        if (std::isnan(BodyMatrix[i])) return true;
    return false;
}
