/* Minimal stand-in for freon::Matrix (not vendored by swegl): storage,
 * row access and the product.  The product sums k = 0..3 left to right; for
 * root nodes (identity parent) every summation order gives the same bits.
 * Test infrastructure for building the reference oracle. */
#pragma once
#include <cstddef>
namespace freon {
template <typename T, std::size_t R, std::size_t C>
struct Matrix {
    T m[R][C];
    T *operator[](std::size_t i) { return m[i]; }
    const T *operator[](std::size_t i) const { return m[i]; }
};
template <typename T, std::size_t R, std::size_t K, std::size_t C>
Matrix<T, R, C> operator*(const Matrix<T, R, K> &a, const Matrix<T, K, C> &b)
{
    Matrix<T, R, C> r;
    for (std::size_t i = 0; i < R; i++)
        for (std::size_t j = 0; j < C; j++) {
            T s = a.m[i][0] * b.m[0][j];
            for (std::size_t k = 1; k < K; k++)
                s = s + a.m[i][k] * b.m[k][j];
            r.m[i][j] = s;
        }
    return r;
}
template <typename T>
struct MatrixIdentity {
    static const Matrix<T, 4, 4> _4;
};
template <typename T>
const Matrix<T, 4, 4> MatrixIdentity<T>::_4 = {{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}}};
} // namespace freon
