// Force-included (g++ -include) ahead of the reference solver's headers when
// the reference's own CPU path is compiled on Linux as the test oracle.
// Written for this project.  It supplies what the MSVC-only reference relies
// on implicitly, without editing any reference file:
//  * standard headers the reference uses without including them
//    (std::vector in KernelConfiguration.h:21-93, std::function in
//    BoundaryConditionConfiguration.h:47, ...);
//  * utility/Direction.h, which utility/Stencil.h uses before declaring it;
//  * replacements for two small utility classes whose reference form only
//    compiles on MSVC.  Both are pre-empted through their include guards and
//    behave the same as the reference on every call the solver makes:
//      - Stencil (utility/Stencil.h:9-66) takes `CellIdx&` and is called with
//        temporaries (ExplicitRungeKuttaFVM.h:367,407,475,516,584,625); the
//        replacement takes `const CellIdx&`;
//      - GradientComputer (utility/GradientComputer.h:9-56) throws
//        `std::exception("...")`, an MSVC-only constructor; the replacement
//        throws std::runtime_error.  It is used only by the viscous path.
#ifndef ORACLE_REF_PRELUDE_HPP
#define ORACLE_REF_PRELUDE_HPP

#include <algorithm>
#include <array>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <valarray>
#include <vector>

#include "utility/Direction.h"
#include "grid.h"

#define TurboStructured_Utility_Stencil
struct CellIdx {
    int i, j, k;
    CellIdx(int _i, int _j, int _k) : i(_i), j(_j), k(_k) {}
};

class Stencil {
    const int nDims;
public:
    const Grid* grid;
    Stencil() : nDims(1), grid(nullptr) {}
    Stencil(int _nDims, Grid& _grid) : nDims(_nDims), grid(&_grid) {}

    // The input cell first, then its neighbours across the two transverse
    // directions (+1 before -1), as utility/Stencil.h:28-63 orders them.
    std::vector<CellIdx> InternalBorderStencil(Direction dir, const CellIdx& c) {
        std::vector<CellIdx> s;
        s.push_back(c);
        auto add_pair = [&s](int di, int dj, int dk, const CellIdx& b) {
            s.push_back(CellIdx(b.i + di, b.j + dj, b.k + dk));
            s.push_back(CellIdx(b.i - di, b.j - dj, b.k - dk));
        };
        if (dir == Direction::XDirection) {
            if (nDims > 1) add_pair(0, 1, 0, c);
            if (nDims > 2) add_pair(0, 0, 1, c);
        } else if (dir == Direction::YDirection) {
            add_pair(1, 0, 0, c);
            if (nDims > 2) add_pair(0, 0, 1, c);
        } else if (dir == Direction::ZDirection) {
            add_pair(1, 0, 0, c);
            add_pair(0, 1, 0, c);
        }
        return s;
    }
};

#include "Vector.h"
#include <Eigen/Dense>

#define TurboStructured_Utility_GradientComputer
class GradientComputer {
    const int nDims;
public:
    GradientComputer() : nDims(1) {}
    GradientComputer(int _nDims) : nDims(_nDims) {}

    // Least-squares gradient from the offsets (point - points[i]) and value
    // differences (value - values[i]) by a thin Jacobi SVD solve.
    Vector ExecuteByLeastSquares(Vector point, double value, const std::vector<Vector>& points,
                                 const std::vector<double>& values) {
        const int m = (int)points.size();
        Eigen::MatrixXd A(m, nDims);
        Eigen::VectorXd rhs(m);
        for (int r = 0; r < m; ++r) {
            Vector d = point - points[r];
            A(r, 0) = d.x;
            if (nDims > 1) A(r, 1) = d.y;
            if (nDims > 2) A(r, 2) = d.z;
            rhs(r) = value - values[r];
        }
        Eigen::JacobiSVD<Eigen::MatrixXd> svd(A, Eigen::ComputeThinU | Eigen::ComputeThinV);
        Eigen::VectorXd x = svd.solve(rhs);
        if (svd.rank() < nDims) throw std::runtime_error("Could not solve for gradient due to rank deficiency");
        Vector g(x(0), 0, 0);
        if (nDims > 1) g.y = x(1);
        if (nDims > 2) g.z = x(2);
        return g;
    }
};

#endif
