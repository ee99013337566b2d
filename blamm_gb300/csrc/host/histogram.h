// histogram.h -- PWM score histograms and the p-value -> threshold inversion.
//
// Same semantics as biointec/blamm's ScoreHistogram (src/motif.h:36-146,
// src/motif.cpp:36-132) and Motif::computeTheoreticalSpectrum
// (src/motif.cpp:151-192), plus the `hist` module (src/hist.cpp).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace blamm {

class Motif;

class ScoreHistogram {
public:
    ScoreHistogram() = default;
    ScoreHistogram(float minScore, float maxScore, size_t numBins);

    // motif.h:96-102 / 109-115: bin = int((score - min) / width), clamped
    void addObservation(float score, uint64_t n = 1);
    void setNumObservations(float score, uint64_t count);  // overwrites the bin
    // motif.cpp:47-69 (double walk from the top bin, float interpolation)
    float scoreCutoff(float pvalue) const;
    // motif.cpp:71-107: <dir><base>.dat (+ .gnu)
    void writeGNUPlotFile(const std::string &dir, const std::string &base, const std::string &label) const;
    // motif.cpp:109-132
    void loadHistogram(const std::string &dir, const std::string &base);

    size_t numBins() const { return counts_.size(); }
    float minScore() const { return min_; }
    float maxScore() const { return max_; }
    float width() const { return width_; }
    const std::vector<uint64_t> &counts() const { return counts_; }
    std::vector<uint64_t> &counts() { return counts_; }

private:
    std::vector<uint64_t> counts_;
    float min_ = 0.0f, max_ = 0.0f, width_ = 0.0f;
};

// Motif::computeTheoreticalSpectrum + Histogram::generateTheoreticalHist:
// fill a histogram with the exact score distribution of a motif under an iid
// background (integerised scores, float DP), maxLength observations.
void theoreticalHistogram(const Motif &m, const std::array<float, 4> &background, size_t maxLength,
                          ScoreHistogram &hist);

// `blamm hist` (hist.cpp:177-266)
int runHistModule(int argc, char **argv);

}  // namespace blamm
