// species.cpp -- see species.h.
#include "species.h"

#include <fstream>
#include <memory>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "blamm_gpu.h"
#include "ingest.h"
#include "sequence.h"

namespace blamm {

void Species::computeNucleotideComposition()
{
    counts_ = {0, 0, 0, 0};
    if (gpuFastaReader()) {
        // the files' text parsed on the GPU piece by piece: counts and header names
        blamm_ctx *ctx = nullptr;
        if (blamm_ctx_create(0, &ctx) != BLAMM_OK)
            throw std::runtime_error("no GPU for the FASTA reader (BLAMM_FASTA_READER=host reads on the host)");
        std::unique_ptr<blamm_ctx, void (*)(blamm_ctx *)> guard(ctx, blamm_ctx_destroy);
        FastaPieceReader rd(sequenceFilenames(), ingestPieceBytes());
        std::string piece;
        seqNames_.clear();
        while (rd.next(piece)) {
            int64_t nb = 0, nr = 0, ns = 0;
            uint64_t c[4] = {0, 0, 0, 0};
            if (blamm_stream_load_fasta(ctx, piece.data(), (int64_t)piece.size(), &nb, &nr, &ns, c) != BLAMM_OK)
                throw std::runtime_error(blamm_last_error(ctx));
            std::vector<int64_t> hp((size_t)ns);
            if (blamm_stream_tables(ctx, nullptr, nullptr, nullptr, hp.data()) != BLAMM_OK)
                throw std::runtime_error(blamm_last_error(ctx));
            for (auto &n : headerNames(piece, hp)) seqNames_.push_back(std::move(n));
            for (int b = 0; b < 4; ++b) counts_[(size_t)b] += c[b];
        }
        totLen_ = counts_[0] + counts_[1] + counts_[2] + counts_[3];
        return;
    }
    FastaStream fs(sequenceFilenames());
    StreamChunk chunk;
    while (fs.nextChunk(chunk, 1 << 24, 0)) {
        for (char c : chunk.bases) {
            switch (c) {
            case 'A': case 'a': ++counts_[0]; break;
            case 'C': case 'c': ++counts_[1]; break;
            case 'G': case 'g': ++counts_[2]; break;
            default: ++counts_[3]; break;  // only T/t reach here
            }
        }
    }
    totLen_ = counts_[0] + counts_[1] + counts_[2] + counts_[3];
    seqNames_ = fs.seqNames();
}

std::array<float, 4> Species::nuclProbabilities(float pseudo) const
{
    float tot = (float)(counts_[0] + counts_[1] + counts_[2] + counts_[3]);
    tot += 4.0f * pseudo;
    std::array<float, 4> p;
    for (int i = 0; i < 4; ++i) p[i] = ((float)counts_[i] + pseudo) / tot;
    return p;
}

void Species::write(std::ostream &os) const
{
    os << "SPECIES" << "\t" << name_ << "\n";
    os << "NUM_FASTA_FILES" << "\t" << files_.size() << "\n";
    for (const auto &f : files_) os << f << "\n";
    os << "TOT_SEQ_LENGTH" << "\t" << totLen_ << "\n";
    os << "NUCL_COUNT_ACGT" << "\t" << counts_[0] << "\t" << counts_[1] << "\t" << counts_[2] << "\t"
       << counts_[3] << "\n";
    os << "NUM_SEQUENCES" << "\t" << seqNames_.size() << "\n";
    for (const auto &s : seqNames_) os << s << "\n";
}

void Species::load(std::istream &is)
{
    std::string tag;
    size_t nfiles = 0, nseq = 0;
    is >> tag >> name_;
    is >> tag >> nfiles;
    for (size_t i = 0; i < nfiles; ++i) {
        is >> tag;
        files_.insert(tag);
    }
    is >> tag >> totLen_;
    is >> tag >> counts_[0] >> counts_[1] >> counts_[2] >> counts_[3];
    is >> tag >> nseq;
    seqNames_.clear();
    seqNames_.reserve(nseq);
    for (size_t i = 0; i < nseq; ++i) {
        is >> tag;
        seqNames_.push_back(tag);
    }
}

void SpeciesContainer::addSeqFile(const std::string &species, const std::string &fasta)
{
    auto it = index_.find(species);
    size_t idx;
    if (it == index_.end()) {
        idx = species_.size();
        index_[species] = idx;
        species_.push_back(Species(species));
    } else {
        idx = it->second;
    }
    species_[idx].addFile(fasta);
}

void SpeciesContainer::computeNucleotideComposition()
{
    for (auto &s : species_) {
        std::cout << "Computing nucleotide composition for " << s.name() << " ...";
        std::cout.flush();
        s.computeNucleotideComposition();
        std::cout << "\n";
    }
}

void SpeciesContainer::write(const std::string &filename) const
{
    std::ofstream ofs(filename.c_str());
    if (!ofs) throw std::runtime_error("Cannot write to file: " + filename);
    ofs << "NUM_SPECIES" << "\t" << species_.size() << "\n";
    for (const auto &s : species_) s.write(ofs);
}

void SpeciesContainer::load(const std::string &filename)
{
    std::ifstream ifs(filename.c_str());
    if (!ifs) throw std::runtime_error("Cannot open file: " + filename);
    std::string tag;
    size_t n = 0;
    ifs >> tag >> n;
    for (size_t i = 0; i < n; ++i) {
        species_.push_back(Species("dummy"));
        species_.back().load(ifs);
        index_[species_.back().name()] = i;
    }
}

Settings::Settings()
{
    std::ifstream ifs("settings.cnf");
    if (!ifs) return;
    defaults = false;
    while (ifs) {
        std::string line, key;
        std::getline(ifs, line);
        if (line.empty() || line[0] == '#') continue;
        std::istringstream iss(line);
        iss >> key;
        if (key == "MATRIX_S_W") iss >> matrix_S_w;
        else if (key == "MATRIX_S_H") iss >> matrix_S_h;
        else if (key == "MATRIX_P_TILE_MIN_ZERO_AREA") iss >> matrix_P_tile_min_zero_area;
        else if (key == "PSEUDOCOUNT") iss >> pseudocount;
        else if (key == "FLUSHOUTPUT") iss >> flushOutput;
        else std::cerr << "WARNING: settings.cnf contains unknown key: " << key << std::endl;
    }
}

void Settings::print() const
{
    if (defaults) std::cout << "File settings.cnf not found, using default values" << std::endl;
    else std::cout << "Loaded configuration from file settings.cnf" << std::endl;
    std::cout << "  MATRIX_S_W = " << matrix_S_w << "; MATRIX_S_H = " << matrix_S_h
              << "; MATRIX_P_TILE_MIN_ZERO_AREA = " << matrix_P_tile_min_zero_area
              << "; PSEUDOCOUNT = " << pseudocount << "; FLUSHOUTPUT = " << flushOutput << "\n";
}

static void dictUsage()
{
    std::cout << "Usage: blamm dict [options] sequences.input\n"
                 "Goal: compute nucleotide frequencies for the input sequences and generate a "
                 "sequence dictionary file\n\n"
                 " [options]\n  -h\t--help\t\tdisplay help message\n\n"
                 " File \"sequences.input\" contains a list of input fasta files in the following format:\n"
                 "   speciesID_1\tspecies1_sequences.fasta\n   ...\n\n"
                 " Example:\n  blamm dict sequences.input\n\n";
}

int runDictModule(int argc, char **argv)
{
    // dict.cpp:53-115
    if (argc < 3) {
        dictUsage();
        exit(EXIT_FAILURE);
    }
    for (int i = 2; i < argc - 1; ++i) {
        const std::string arg(argv[i]);
        dictUsage();
        exit(arg == "-h" || arg == "--help" ? EXIT_SUCCESS : EXIT_FAILURE);
    }
    std::cout << "Welcome to blamm -- dictionary model" << std::endl;
    const std::string manifest(argv[argc - 1]);
    std::ifstream ifs(manifest.c_str());
    if (!ifs) throw std::runtime_error("Could not open file: " + manifest);
    SpeciesContainer sc;
    while (ifs) {
        std::string line, sp, fa;
        std::getline(ifs, line);
        if (line.empty()) continue;
        std::istringstream iss(line);
        iss >> sp >> fa;
        if (sp.empty() || fa.empty())
            throw std::runtime_error("File " + manifest +
                                     " has incorrect format.\nRefer to the documention for more information.");
        std::ifstream fn(fa);
        if (!fn) throw std::runtime_error("Could not open fasta file: " + fa);
        sc.addSeqFile(sp, fa);
    }
    sc.computeNucleotideComposition();
    sc.write(manifest + ".dict");
    std::cout << "Done!  Dictionary written to " << manifest + ".dict" << std::endl;
    return 0;
}

}  // namespace blamm
