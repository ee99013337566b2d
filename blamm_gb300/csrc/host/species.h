// species.h -- sequence groups ("species"), the .dict file, settings.cnf.
//
// Same semantics and file formats as biointec/blamm's Species /
// SpeciesContainer (src/species.h, src/species.cpp), Settings
// (src/settings.cpp) and the `dict` module (src/dict.cpp).
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <vector>

namespace blamm {

class Species {
public:
    explicit Species(std::string name = "dummy") : name_(std::move(name)) {}
    const std::string &name() const { return name_; }
    void addFile(const std::string &f) { files_.insert(f); }
    // std::set order (byte-wise sorted), as the reference reads them
    std::vector<std::string> sequenceFilenames() const { return {files_.begin(), files_.end()}; }
    const std::array<uint64_t, 4> &nuclCounts() const { return counts_; }
    uint64_t totalSeqLength() const { return totLen_; }
    const std::vector<std::string> &seqNames() const { return seqNames_; }
    const std::string &seqName(size_t i) const { return seqNames_[i]; }

    // species.cpp:32-61 (ACGT counts over the filtered stream, case-insensitive)
    void computeNucleotideComposition();
    // species.cpp:63-71
    std::array<float, 4> nuclProbabilities(float pseudo) const;
    void write(std::ostream &os) const;
    void load(std::istream &is);

private:
    std::string name_;
    std::set<std::string> files_;
    std::array<uint64_t, 4> counts_{{0, 0, 0, 0}};
    uint64_t totLen_ = 0;
    std::vector<std::string> seqNames_;
};

class SpeciesContainer {
public:
    void addSeqFile(const std::string &species, const std::string &fasta);
    void computeNucleotideComposition();
    void write(const std::string &filename) const;
    void load(const std::string &filename);
    size_t size() const { return species_.size(); }
    const Species &operator[](size_t i) const { return species_[i]; }
    std::vector<Species>::const_iterator begin() const { return species_.begin(); }
    std::vector<Species>::const_iterator end() const { return species_.end(); }

private:
    std::vector<Species> species_;
    std::map<std::string, size_t> index_;
};

struct Settings {
    // settings.cpp:481-521: read settings.cnf from the working directory
    Settings();
    void print() const;
    size_t matrix_S_w = 250, matrix_S_h = 1000, matrix_P_tile_min_zero_area = 64 * 64,
           flushOutput = 100000;
    float pseudocount = 0.25f;
    bool defaults = true;
};

int runDictModule(int argc, char **argv);

}  // namespace blamm
