// motif.h -- motifs, PWMs and the motif matrix P (host side of the scan).
//
// Same semantics as biointec/blamm's Motif / MotifContainer (src/motif.h,
// src/motif.cpp): JASPAR and Cluster-Buster parsing, length sort, reverse
// complements, PFM -> PWM conversion in float, the zero-padded column-major
// P, min/max scores and the P tiling printout.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace blamm {

class Motif {
public:
    Motif() = default;
    explicit Motif(std::string name) : name_(std::move(name)) {}

    const std::string &name() const { return name_; }
    size_t size() const { return pfm_.size(); }
    bool isRevCompl() const { return revcomp_; }
    float threshold() const { return threshold_; }
    void setThreshold(float t) { threshold_ = t; }
    void addCharacter(const std::array<uint64_t, 4> &c) { pfm_.push_back(c); }
    const std::vector<std::array<uint64_t, 4>> &pfm() const { return pfm_; }
    const std::array<float, 4> &operator[](size_t i) const { return pwm_[i]; }
    const std::vector<std::array<float, 4>> &pwm() const { return pwm_; }

    // Motif::PFM2PWM (motif.cpp:194-223): log2 of (count+pc)/(total+4pc) over
    // the background probability, in float; reverse-complement motifs use the
    // complemented background.
    void pfm2pwm(const std::array<uint64_t, 4> &bgCounts, float pseudo);
    // Motif::revCompl (motif.cpp:267-286)
    void revCompl();
    float maxScore() const;  // motif.cpp:241-252
    float minScore() const;  // motif.cpp:254-265
    // base name without a "__<digits>" permutation suffix (motif.h:256-267)
    std::string baseName() const;
    bool isPermutation() const;  // motif.h:273-281

    bool operator<(const Motif &rhs) const { return size() < rhs.size(); }

private:
    std::string name_;
    std::vector<std::array<uint64_t, 4>> pfm_;
    std::vector<std::array<float, 4>> pwm_;
    float threshold_ = 0.0f;
    bool revcomp_ = false;
};

struct MatrixTile {
    size_t rowStart, colStart, rowEnd, colEnd;
};

class MotifContainer {
public:
    // MotifContainer::load (motif.cpp:323-338): ".jaspar" suffix -> JASPAR,
    // anything else Cluster-Buster; sorted by length with std::sort.
    void load(const std::string &filename, bool loadPermutations);
    void addReverseComplements();  // motif.cpp:439-449: [m0, rc(m0), m1, rc(m1), ...]
    // motif.cpp:542-564: PWMs for a background and the column-major P (4*Lmax rows)
    void generateMatrix(const std::array<uint64_t, 4> &bgCounts, float pseudo);
    // motif.cpp:482-540 (greedy length split); used for the console report
    void generateMatrixTiles(size_t tileMinZeroArea, bool verbose);

    size_t size() const { return motifs_.size(); }
    size_t maxMotifLen() const;
    Motif &operator[](size_t i) { return motifs_[i]; }
    const Motif &operator[](size_t i) const { return motifs_[i]; }
    std::vector<Motif>::iterator begin() { return motifs_.begin(); }
    std::vector<Motif>::iterator end() { return motifs_.end(); }
    const std::vector<float> &matrix() const { return P_; }  // column-major
    size_t matrixRows() const { return rows_; }
    const std::vector<MatrixTile> &tiles() const { return tiles_; }

private:
    std::vector<Motif> motifs_;
    std::vector<float> P_;
    size_t rows_ = 0;
    std::vector<MatrixTile> tiles_;
};

}  // namespace blamm
