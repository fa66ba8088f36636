// Host side of trimesh::transform (corelib/src/geometry.cpp:76-87): the normal matrix
// ~(T ^ -1) in the reference's float arithmetic.
//
// mat::operator^(-1) (corelib/src/tensor.h:511-540) inverts a 4x4 matrix as adjugate / det, the
// adjugate by cofactors whose minors are expanded along successive columns over the remaining
// rows in increasing order, each expansion summed into a float from 0 in that order
// (tensor.h:451-509); det(adj) sums a(i, 0) * adj(0, i) over i; the inverse is (1 / det) * adj,
// and a |det| <= 1e-5 is "not invertible" (tensor.h:16, :524). The expansion below visits the
// same terms in the same order, so the normals come out bit for bit as the reference's.
#include "scene_pack.h"

#include <cmath>

namespace e8g {
namespace {

// Determinant of the submatrix of a on the rows in `rows` (bit r = row r) and the columns
// cols[0..k), k = number of rows, by expansion along cols[0].
float cofactor_det(float const a[4][4], unsigned rows, int const *cols) {
    int first = 0;
    while (!(rows >> first & 1))
        first++;
    if ((rows & (rows - 1)) == 0)
        return a[first][cols[0]];
    float d = 0.0f;
    int pos = 0;
    for (int r = 0; r < 4; r++) {
        if (!(rows >> r & 1))
            continue;
        float minor = cofactor_det(a, rows & ~(1u << r), cols + 1);
        float x = a[r][cols[0]];
        d += (pos & 1 ? -x : x) * minor;
        pos++;
    }
    return d;
}

} // namespace

bool reference_normal_matrix(float const m[16], float n_out[16]) {
    float a[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            a[i][j] = m[4 * i + j];
    float adj[4][4];
    for (int j = 0; j < 4; j++) {     // column removed
        int cols[3], k = 0;
        for (int c = 0; c < 4; c++)
            if (c != j)
                cols[k++] = c;
        for (int i = 0; i < 4; i++) { // row removed
            float minor = cofactor_det(a, 0xFu & ~(1u << i), cols);
            adj[j][i] = ((i + j) & 1) ? -minor : minor;
        }
    }
    float det = 0;
    for (int i = 0; i < 4; i++)
        det += a[i][0] * adj[0][i];
    if (std::fabs(det - 0.0f) <= 1e-5f)
        return false;
    float k = 1.0f / det;
    // inverse(i, j) = k * adj(i, j); the normal matrix is its transpose
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            n_out[4 * i + j] = k * adj[j][i];
    return true;
}

} // namespace e8g
