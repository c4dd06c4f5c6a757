/**
 * @file senk_blas2.hpp
 * @brief senk::blas2::Trsv (reference include/senk_blas2.hpp:24-34): the m×m
 * back substitution of GMRES's least-squares problem. It acts on a few dozen
 * scalars and stays on the host; the GPU solvers do the same step on the device.
 */
#ifndef SENK_BLAS2_HPP
#define SENK_BLAS2_HPP

namespace senk {

namespace blas2 {

/** x = U⁻¹ b for the leading m×m upper triangle of U (column-major, ld n). */
template <typename T>
void Trsv(T *U, T *b, T *x, int n, int m)
{
    for (int i = m - 1; i >= 0; i--) {
        T t = b[i];
        for (int j = m - 1; j > i; j--) t -= U[j * n + i] * x[j];
        x[i] = t / U[i * n + i];
    }
}

}  // namespace blas2

}  // namespace senk

#endif
