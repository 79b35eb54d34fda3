// Minimal stand-in for the three deal.II value types that the reference's mesh and
// interpolator sources name in their headers (Point<3>, Tensor<1,3>, CellData<3>).
// It lets those sources compile without deal.II so that their own mesh-split, cell
// precompute, point-location and interpolation code can be run as a test oracle.
// Nothing here computes anything; it only carries three doubles or eight indices.
#ifndef FEMOCS_GB300_ORACLE_DEALII_STUB_H
#define FEMOCS_GB300_ORACLE_DEALII_STUB_H

#include <array>
#include <vector>
#include <map>
#include <string>
#include <cmath>
#include <algorithm>
#include <iostream>
#include <sstream>
#include <fstream>
#include <iomanip>

namespace dealii {

template <int dim, typename Number = double>
class Point {
public:
    Point() { v.fill(0); }
    Point(Number x, Number y, Number z) { v[0] = x; v[1] = y; v[2] = z; }
    Number operator[](int i) const { return v[i]; }
    Number& operator[](int i) { return v[i]; }
private:
    std::array<Number, 3> v;
};

template <int rank, int dim, typename Number = double>
class Tensor {
public:
    Tensor() { v.fill(0); }
    Number operator[](int i) const { return v[i]; }
    Number& operator[](int i) { return v[i]; }
private:
    std::array<Number, 3> v;
};

template <int dim>
struct CellData {
    unsigned int vertices[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int material_id = 0;
};

}  // namespace dealii

#endif
