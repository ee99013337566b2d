// histogram.cpp -- see histogram.h.
#include "histogram.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <thread>

#include "motif.h"
#include "species.h"

namespace blamm {

ScoreHistogram::ScoreHistogram(float minScore, float maxScore, size_t numBins)
    : counts_(numBins, 0), min_(minScore), max_(maxScore)
{
    width_ = (maxScore - minScore) / (float)numBins;
}

static int binOf(float score, float min, float width, size_t nbins)
{
    int b = int((score - min) / width);
    b = std::max<int>(0, b);
    b = std::min<int>((int)nbins - 1, b);
    return b;
}

void ScoreHistogram::addObservation(float score, uint64_t n)
{
    counts_[binOf(score, min_, width_, counts_.size())] += n;
}

void ScoreHistogram::setNumObservations(float score, uint64_t count)
{
    counts_[binOf(score, min_, width_, counts_.size())] = count;
}

float ScoreHistogram::scoreCutoff(float pvalue) const
{
    double tot = 0.0;
    for (uint64_t c : counts_) tot += (double)c;
    double curr = pvalue * tot;
    for (long i = (long)counts_.size() - 1; i >= 0; --i) {
        if ((double)counts_[i] < curr) {
            curr -= (double)counts_[i];
        } else {
            const double frac = curr / (double)counts_[i];
            const float cutoffi = (float)(frac * i + (1.0 - frac) * (i + 1));
            return cutoffi * width_ + min_;
        }
    }
    return max_;
}

void ScoreHistogram::writeGNUPlotFile(const std::string &dir, const std::string &base,
                                      const std::string &label) const
{
    std::string fn = dir + base + ".dat";
    std::ofstream ofs(fn.c_str());
    if (!ofs) throw std::runtime_error("Error: cannot write to file " + fn);
    ofs << counts_.size() << "\t" << min_ << "\t" << max_ << "\n";
    for (size_t i = 0; i < counts_.size(); ++i)
        ofs << (0.5 + i) * width_ + min_ << "\t" << counts_[i] << "\n";
    ofs.close();
    uint64_t maxy = 0;
    for (uint64_t c : counts_) maxy = std::max(maxy, c);
    maxy = (uint64_t)((double)maxy * 1.1);
    fn = dir + base + ".gnu";
    ofs.open(fn.c_str());
    if (!ofs) throw std::runtime_error("Error: cannot write to file " + fn);
    ofs << "set output \"" << base << ".ps\"\n";
    ofs << "set key autotitle columnhead\n";
    ofs << "set terminal postscript landscape\n";
    ofs << "set terminal postscript noenhanced\n";
    ofs << "set xrange [" << min_ << ":" << max_ << "]\n";
    ofs << "set yrange [" << 0 << ":" << maxy << "]\n";
    ofs << "set xlabel 'PWM score'" << std::endl;
    ofs << "set ylabel 'count'" << std::endl;
    ofs << "plot \"" << base << ".dat\" using 1:2 title '" << label << "' with boxes\n";
}

void ScoreHistogram::loadHistogram(const std::string &dir, const std::string &base)
{
    const std::string fn = dir + base + ".dat";
    std::ifstream ifs(fn.c_str());
    if (!ifs) throw std::runtime_error("Error: cannot read file " + fn + ". Did you run the hist module?");
    size_t nbins = 0;
    ifs >> nbins >> min_ >> max_;
    width_ = (max_ - min_) / (float)nbins;
    counts_.assign(nbins, 0);
    for (size_t i = 0; i < nbins; ++i) {
        float bin;
        uint64_t v;
        ifs >> bin >> v;
        counts_[i] = v;
    }
    if (!ifs) throw std::runtime_error("Unexpected end-of-file reached");
}

void theoreticalHistogram(const Motif &m, const std::array<float, 4> &background, size_t maxLength,
                          ScoreHistogram &hist)
{
    // motif.cpp:151-192: integerise a*PWM+b, DP over positions in float with
    // ordered maps (the insertion order of the float sums matters)
    const size_t L = m.size();
    if (L == 0) return;
    const float minS = m.minScore(), maxS = m.maxScore();
    const float range = maxS - minS;
    const float a = (float)hist.numBins() / range;
    const float b = -a * minS / (float)L;
    std::vector<std::array<int, 4>> q(L);
    for (size_t p = 0; p < L; ++p)
        for (int k = 0; k < 4; ++k) q[p][k] = (int)std::round(a * m[p][k] + b);
    std::map<int, float> cur, nxt;
    for (int k = 0; k < 4; ++k) cur[q[0][k]] += background[k];
    for (size_t p = 1; p < L; ++p) {
        nxt.clear();
        for (const auto &it : cur)
            for (int k = 0; k < 4; ++k) nxt[it.first + q[p][k]] += it.second * background[k];
        std::swap(cur, nxt);
    }
    std::map<float, float> spectrum;
    for (const auto &it : cur) spectrum.insert(std::make_pair(((float)it.first - L * b) / a, it.second));
    for (const auto &it : spectrum) hist.setNumObservations(it.first, maxLength * it.second);
}

// ------------------------------------------------------------------ module
static void histUsage()
{
    std::cout << "Usage: blamm hist [options] motifs.input sequences.input\n"
                 "Goal: compute PWM score histograms\n\n"
                 " [options]\n"
                 "  -e\t--empirical\tcompute empirical histograms\n"
                 "  -h\t--help\t\tdisplay help message\n\n"
                 " [options arg]\n"
                 "  -b\t--numbins\tnumber of bins per histogram [default = 250]\n"
                 "  -t\t--numthreads\tset the number of parallel threads [default = #cores]\n"
                 "  -l\t--length\tlength of sequence data to analyze [default = 10000000]\n\n"
                 " [file_options]\n"
                 "  -H\t--histdir\toutput directory for the histogram file(s) [default = .]\n\n"
                 " Example:\n  blamm hist motifs.input sequences.input\n\n";
}

// empirical histograms are computed on the GPU (scan.cpp)
void empiricalHistograms(const Species &species, MotifContainer &motifs, size_t maxLength,
                         std::vector<ScoreHistogram> &hists);

int runHistModule(int argc, char **argv)
{
    if (argc < 4) {
        histUsage();
        exit(EXIT_FAILURE);
    }
    size_t maxLength = 10000000, numBins = 250;
    bool empirical = false;
    std::string histdir;
    size_t numThreads = std::thread::hardware_concurrency();
    for (int i = 2; i < argc - 2; ++i) {
        const std::string arg(argv[i]);
        if (arg == "-h" || arg == "--help") {
            histUsage();
            exit(EXIT_SUCCESS);
        } else if ((arg == "-l" || arg == "--length") && i + 1 < argc - 2) {
            maxLength = std::atoll(argv[++i]);
        } else if ((arg == "-b" || arg == "--numbins") && i + 1 < argc - 2) {
            numBins = std::atoll(argv[++i]);
            if (numBins < 2) numBins = 2;
        } else if (arg == "-e" || arg == "--empirical") {
            empirical = true;
        } else if ((arg == "-t" || arg == "--numthreads") && i + 1 < argc - 2) {
            numThreads = std::atoi(argv[++i]);
        } else if ((arg == "-H" || arg == "--histdir") && i + 1 < argc - 2) {
            histdir = argv[++i];
            if (histdir.back() != '/') histdir.push_back('/');
        } else {
            histUsage();
            exit(EXIT_FAILURE);
        }
    }
    (void)numThreads;
    Settings settings;
    std::cout << "Welcome to blamm -- histogram module" << std::endl;
    SpeciesContainer species;
    species.load(std::string(argv[argc - 1]) + ".dict");
    MotifContainer motifs;
    motifs.load(argv[argc - 2], false);
    std::cout << "Loaded " << motifs.size() << " motifs from disk";
    std::cout << "\nMaximum motif size: " << motifs.maxMotifLen() << std::endl;
    for (const auto &sp : species) {
        std::cout << "Generating histograms for species: " << sp.name() << std::endl;
        motifs.generateMatrix(sp.nuclCounts(), settings.pseudocount);
        std::vector<ScoreHistogram> hists;
        for (size_t i = 0; i < motifs.size(); ++i)
            hists.emplace_back(motifs[i].minScore(), motifs[i].maxScore(), numBins);
        if (empirical) {
            empiricalHistograms(sp, motifs, maxLength, hists);
        } else {
            const auto bg = sp.nuclProbabilities(settings.pseudocount);
            for (size_t i = 0; i < motifs.size(); ++i) theoreticalHistogram(motifs[i], bg, maxLength, hists[i]);
        }
        for (size_t i = 0; i < hists.size(); ++i)
            hists[i].writeGNUPlotFile(histdir, "hist_" + sp.name() + "_" + motifs[i].name(),
                                      motifs[i].name() + " (" + sp.name() + ")");
    }
    return 0;
}

}  // namespace blamm
