// Read access to the unit-interval mass and stiffness matrices that
// Grid::getMass() / Grid::getStiff() return (cppsrc/Grid.h:46-47).
//
// The reference's Matrix (cppsrc/Matrix.h:70-117) is a general dense matrix
// with arithmetic and a QR solver used inside its element operators.  Here
// the operators run on the GPU, so this class keeps only its read accessors:
// rows(), cols(), row pointers through operator[] (zero-based) and the
// one-based operator()(row, col).  It holds a copy of the matrices the
// simulation was created with (matrices.txt or the generated ones).
#pragma once

#include <vector>

class Matrix {
public:
    Matrix() = default;
    Matrix(unsigned rows, unsigned cols, const double* data)
        : mRows(rows), mCols(cols), mData(data, data + (size_t)rows * cols)
    {
    }
    unsigned rows() const { return mRows; }
    unsigned cols() const { return mCols; }
    const double* operator[](unsigned row) const { return mData.data() + (size_t)row * mCols; }
    double operator()(unsigned row, unsigned col) const { return mData[(size_t)(row - 1) * mCols + (col - 1)]; }

private:
    unsigned mRows = 0, mCols = 0;
    std::vector<double> mData;
};
