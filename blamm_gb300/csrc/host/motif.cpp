// motif.cpp -- see motif.h.
#include "motif.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <iostream>
#include <numeric>
#include <sstream>
#include <stdexcept>

namespace blamm {

void Motif::pfm2pwm(const std::array<uint64_t, 4> &bgCounts, float pseudo)
{
    float bgTot = (float)(bgCounts[0] + bgCounts[1] + bgCounts[2] + bgCounts[3]);
    bgTot += 4.0f * pseudo;
    std::array<float, 4> bg;
    for (int i = 0; i < 4; ++i) bg[i] = ((float)bgCounts[i] + pseudo) / bgTot;
    if (revcomp_) {
        std::swap(bg[0], bg[3]);
        std::swap(bg[1], bg[2]);
    }
    pwm_.resize(pfm_.size());
    for (size_t i = 0; i < pfm_.size(); ++i) {
        float tot = (float)(pfm_[i][0] + pfm_[i][1] + pfm_[i][2] + pfm_[i][3]);
        tot += 4.0f * pseudo;
        for (int j = 0; j < 4; ++j) {
            const float ppm = ((float)pfm_[i][j] + pseudo) / tot;
            pwm_[i][j] = std::log2(ppm / bg[j]);
        }
    }
}

void Motif::revCompl()
{
    std::reverse(pfm_.begin(), pfm_.end());
    for (auto &c : pfm_) c = {c[3], c[2], c[1], c[0]};
    std::reverse(pwm_.begin(), pwm_.end());
    for (auto &c : pwm_) c = {c[3], c[2], c[1], c[0]};
    revcomp_ = !revcomp_;
}

float Motif::maxScore() const
{
    float s = 0.0f;
    for (const auto &p : pwm_) s += std::max(std::max(p[0], p[1]), std::max(p[2], p[3]));
    return s;
}

float Motif::minScore() const
{
    float s = 0.0f;
    for (const auto &p : pwm_) s += std::min(std::min(p[0], p[1]), std::min(p[2], p[3]));
    return s;
}

static long permutationSplit(const std::string &name)
{
    long i = (long)name.size() - 1;
    while (i >= 0 && std::isdigit((unsigned char)name[i])) --i;
    if (i < 1) return -1;
    return (name[i - 1] == '_' && name[i] == '_') ? i - 1 : -1;
}

std::string Motif::baseName() const
{
    const long s = permutationSplit(name_);
    return s < 0 ? name_ : name_.substr(0, (size_t)s);
}

bool Motif::isPermutation() const { return permutationSplit(name_) >= 0; }

// ------------------------------------------------------------------ loading
static void loadJaspar(const std::string &filename, std::vector<Motif> &out)
{
    std::ifstream ifs(filename.c_str());
    if (!ifs) throw std::runtime_error("Could not open file: " + filename);
    while (ifs.good()) {
        std::string name, rest;
        ifs >> name;
        if (!name.empty()) name = name.substr(1);
        std::getline(ifs, rest);
        if (!ifs) break;
        std::vector<std::vector<uint64_t>> freq(4);
        for (int i = 0; i < 4; ++i) {
            std::string line, tok;
            std::getline(ifs, line);
            std::istringstream iss(line);
            iss >> tok >> tok;  // letter and '['
            uint64_t v;
            while (iss >> v) freq[i].push_back(v);
        }
        Motif m(name);
        for (size_t j = 0; j < freq[0].size(); ++j) {
            std::array<uint64_t, 4> c{};
            for (int k = 0; k < 4; ++k) c[k] = j < freq[k].size() ? freq[k][j] : 0;
            m.addCharacter(c);
        }
        out.push_back(m);
    }
    std::sort(out.begin(), out.end());
}

static void loadClusterBuster(const std::string &filename, std::vector<Motif> &out)
{
    std::ifstream ifs(filename.c_str());
    if (!ifs) throw std::runtime_error("Could not open file: " + filename);
    while (ifs.good()) {
        std::string line;
        std::getline(ifs, line);
        if (line.empty()) continue;
        if (line.front() == '>') {
            out.push_back(Motif(line.substr(1)));
            continue;
        }
        if (out.empty()) throw std::runtime_error("Incorrect motif file format: " + filename);
        std::istringstream iss(line);
        uint64_t a = 0, c = 0, g = 0, t = 0;
        iss >> a >> c >> g >> t;
        out.back().addCharacter({a, c, g, t});
    }
    std::sort(out.begin(), out.end());
}

void MotifContainer::load(const std::string &filename, bool loadPermutations)
{
    std::vector<Motif> all;
    if (filename.size() > 7 && filename.substr(filename.size() - 7) == ".jaspar")
        loadJaspar(filename, all);
    else
        loadClusterBuster(filename, all);
    for (auto &m : all)
        if (loadPermutations || !m.isPermutation()) motifs_.push_back(m);
}

void MotifContainer::addReverseComplements()
{
    std::vector<Motif> fwd = motifs_;
    motifs_.clear();
    for (auto &m : fwd) {
        motifs_.push_back(m);
        m.revCompl();
        motifs_.push_back(m);
    }
}

size_t MotifContainer::maxMotifLen() const
{
    size_t l = 0;
    for (const auto &m : motifs_) l = std::max(l, m.size());
    return l;
}

void MotifContainer::generateMatrix(const std::array<uint64_t, 4> &bgCounts, float pseudo)
{
    for (auto &m : motifs_) m.pfm2pwm(bgCounts, pseudo);
    rows_ = 4 * maxMotifLen();
    P_.assign(rows_ * motifs_.size(), 0.0f);
    for (size_t c = 0; c < motifs_.size(); ++c)
        for (size_t j = 0; j < motifs_[c].size(); ++j)
            for (int b = 0; b < 4; ++b) P_[c * rows_ + 4 * j + b] = motifs_[c][j][b];
}

void MotifContainer::generateMatrixTiles(size_t minZeroArea, bool verbose)
{
    const size_t nRows = 4 * maxMotifLen(), nCols = motifs_.size();
    if (verbose) std::cout << "Matrix P has dimensions: " << nRows << " x " << nCols << std::endl;
    tiles_.assign(1, MatrixTile{0, 0, nRows, nCols});
    if (nCols == 0) return;
    for (bool split = true; split;) {
        split = false;
        std::vector<MatrixTile> next;
        for (const auto &t : tiles_) {
            // findBestSplit (motif.cpp:451-471): the cut maximising the zero area removed
            size_t best = 0, bestJ = t.colStart + 1;
            for (size_t j = t.colStart + 1; j < t.colEnd; ++j) {
                const size_t area = (j - t.colStart) * (t.rowEnd - 4 * motifs_[j - 1].size());
                if (area > best) {
                    best = area;
                    bestJ = j;
                }
            }
            const MatrixTile left{t.rowStart, t.colStart, 4 * motifs_[bestJ - 1].size(), bestJ};
            const MatrixTile right{t.rowStart, bestJ, t.rowEnd, t.colEnd};
            // keepSplit (motif.cpp:473-480)
            if (minZeroArea > 0 && (right.rowEnd - left.rowEnd) * (left.colEnd - left.colStart) >= minZeroArea) {
                next.push_back(left);
                next.push_back(right);
                split = true;
            } else {
                next.push_back(t);
            }
        }
        tiles_ = next;
    }
    if (!verbose) return;
    size_t zeros = 0;
    for (size_t i = 0; i < nCols; ++i) zeros += nRows - 4 * motifs_[i].size();
    const auto prec = std::cout.precision();
    std::cout.precision(2);
    std::cout << "Matrix P initially contains " << 100.0 * (double)zeros / (double)(nRows * nCols)
              << "% zeros\n";
    std::cout << "Matrix P has been partitioned into " << tiles_.size() << " tile(s):\n";
    for (const auto &t : tiles_)
        std::cout << "\tmotif [" << t.colStart << " - " << t.colEnd << "[ -- max. length = " << t.rowEnd
                  << "\n";
    for (const auto &t : tiles_) zeros -= (nRows - t.rowEnd) * (t.colEnd - t.colStart);
    std::cout << "Tiled matrix P contains " << 100.0 * (double)zeros / (double)(nRows * nCols) << "% zeros\n";
    std::cout.precision(prec);
}

}  // namespace blamm
