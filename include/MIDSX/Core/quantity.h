// quantity.h - measured values of the MIDSX C++ API (reference: include/MIDSX/Core/quantity.h).
//
// The reference's VectorValue keeps every sample (src/MIDSX/Core/quantity.cpp:3-94).  On the
// GPU path tallies accumulate (count, sum, sum of squares) per class, which is all the
// reference's statistics use; VectorValue therefore holds that summary.  Samples added on the
// host with addValue/addValues are also kept, so getVector() works for them; a value filled
// from the device is summary-only and getVector() throws std::logic_error.
#pragma once
#include <cmath>
#include <stdexcept>
#include <vector>

class VectorValue {
public:
    VectorValue operator+(VectorValue& other) const;

    void addValue(double value);
    void addValues(const std::vector<double>& values);
    // Adds a block of samples given by its summary (count, sum, sum of squares).
    void addSummary(double count, double sum, double sum_of_squares);

    std::vector<double>& getVector();
    double getSum();
    double getSumSTD();    // sqrt(n * sample variance), src/MIDSX/Core/quantity.cpp:37-45
    double getMean();
    double getMeanSTD();   // sqrt(sample variance / n)
    double getCount();
    double getCountSTD();  // sqrt(n)
    double getVariance();  // sample variance (n - 1 denominator)
    double getSumOfSquares() const { return sumsq_; }
    bool isSummaryOnly() const { return summary_only_; }

private:
    std::vector<double> values_;
    double n_ = 0, sum_ = 0, sumsq_ = 0;
    bool summary_only_ = false;
};

class CountValue {
public:
    CountValue operator+(const CountValue& other) const;
    void addCount();
    void addCounts(long long count);
    long long getCount() const;
    double getCountSTD() const;

    long long count_ = 0;
};
