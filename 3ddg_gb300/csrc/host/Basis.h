// The reference's Basis class surface (cppsrc/Basis.h:19-40): LGL zeros and
// weights per order read from the coefficient files, plus the derivative
// matrix file.  Backed by the package's FP64 basis module.
#pragma once

#include <string>
#include <vector>

using std::string;
using std::vector;

class Basis {
public:
    // Reads hardcoded_coeff.txt / hardcoded_coeff2.txt like the reference
    // (cppsrc/Basis.cpp:74-237); throws std::runtime_error with the reference's
    // message when a file cannot be opened.
    Basis(string filename, string filename2);
    // Generates the same tables from LGL mathematics (no files).
    explicit Basis(int kmax = 10);

    vector<double>* getZeros(unsigned short int order) { return &mZeros[order]; }
    vector<double>* getWeights(unsigned short int order) { return &mWeights[order]; }
    vector<vector<double>>* getDPsi(unsigned short int order) { return &mDPsi[order]; }
    vector<vector<double>>* getPsi(unsigned short int order) { return &mPsi[order]; }

    // Path of the coefficient file this basis was read from ("" if generated).
    const string& coeffFile() const { return mCoeffFile; }

private:
    void load(const string& filename, const string& filename2);
    vector<vector<vector<double>>> mPsi;
    vector<vector<vector<double>>> mDPsi;
    vector<vector<double>> mZeros;
    vector<vector<double>> mWeights;
    string mCoeffFile;
};
