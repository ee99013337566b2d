// scan.cpp -- `blamm scan`: the drop-in PWMScan module driving libblamm_gpu.
//
// Same command line, thresholds, PWMthresholds.txt and occurrence format as
// biointec/blamm's PWMScan (src/pwmscan.cpp:456-648, 81-102).  The BLAS /
// cuBLAS block loop (scanThreadBLAS / scanThreadCUBLAS, :223-437) is replaced
// by: a reader thread that streams FASTA into large overlapping chunks, one
// worker per GPU that scans a chunk with one blamm_scan call (fused tcgen05
// kernel), and a formatter that maps stream positions to (sequence, position)
// and writes the lines.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <vector>

#include "blamm_gpu.h"
#include "format.h"
#include "histogram.h"
#include "ingest.h"
#include "motif.h"
#include "sequence.h"
#include "species.h"

namespace blamm {

namespace {

void scanUsage()
{
    std::cout << "Usage: blamm scan [options] motifs.input sequences.input\n"
                 "Goal: find PWM matches in sequences\n\n"
                 " [options]\n"
                 "  -h\t--help\t\tdisplay help message\n"
                 "  -s\t--simple\tscore lowercase bases too (the simple scan algorithm's scores)\n"
                 "  -c\t--cuda\t\tenable the CUDA scan algorithm (always on)\n"
                 "  -rc\t--revcompl\talso search the reverse strand for occurrences\n\n"
                 " [options arg]\n"
                 "  -at\t--absthreshold\tset the minimal absolute score for a motif occurrence\n"
                 "  -rt\t--relthreshold\tset the minimal relative score [0..1] for a motif occurrence "
                 "(default = 0.95)\n"
                 "  -pt\t--pthreshold\tcompute the motif score threshold from p-value [0..1] (default = 1E-4)\n"
                 "  -t\t--numthreads\tset the number of parallel threads [default = #cores]\n"
                 "  -m\t--mode\t\tGPU arithmetic: auto (default), bf16x2, bf16, e4m3 or fp32\n\n"
                 " [file_options]\n"
                 "  -H\t--histdir\tdirectory where the histogram file(s) are stored [default = .]\n"
                 "  -o\t--output\tfilename for the motif occurrences [default = occurences.txt]\n\n"
                 " Example:\n  blamm scan -o occurences.txt motifs.input sequences.input\n\n";
}

struct Options {
    bool simple = false, revCompl = false;
    bool absSet = false, relSet = false, pSet = false;
    float absThreshold = 0.0f, relThreshold = 0.95f, pvalue = 0.0001f;
    size_t numThreads = std::max(1u, std::thread::hardware_concurrency());
    std::string histdir, output = "occurrences.txt";
    int mode = BLAMM_MODE_AUTO;
};

// One GPU context per device (the reference runs one host thread per device,
// pwmscan.cpp:439-453).
struct Device {
    blamm_ctx *ctx = nullptr;
    std::vector<blamm_hit> hits;
};

void check(blamm_ctx *ctx, int rc, const char *what)
{
    if (rc != BLAMM_OK)
        throw std::runtime_error(std::string("GPU error in ") + what + ": " + blamm_last_error(ctx));
}

// scan one chunk on one device, growing the hit buffer on overflow: the chunk's bases from
// host memory, or (resident) positions [chunk.offset, chunk.offset + size) of the device's
// resident stream
void scanChunk(Device &dev, const StreamChunk &chunk, bool resident = false, int64_t size = 0)
{
    const std::vector<int64_t> runs = chunk.runStarts();
    if (dev.hits.empty()) dev.hits.resize(1 << 20);
    while (true) {
        int64_t nh = 0;
        const int rc = resident
            ? blamm_scan_stream(dev.ctx, chunk.offset, size, runs.data(), (int64_t)runs.size(), dev.hits.data(),
                                (int64_t)dev.hits.size(), &nh)
            : blamm_scan(dev.ctx, chunk.bases.data(), (int64_t)chunk.bases.size(), runs.data(),
                         (int64_t)runs.size(), dev.hits.data(), (int64_t)dev.hits.size(), &nh);
        if (rc == BLAMM_ERR_OVERFLOW) {
            dev.hits.resize((size_t)(nh + nh / 8 + 1024));
            continue;
        }
        check(dev.ctx, rc, resident ? "blamm_scan_stream" : "blamm_scan");
        dev.hits.resize((size_t)nh);  // hits beyond nh were never written
        return;
    }
}

using Clock = std::chrono::steady_clock;

// Wall time per pipeline phase (summed over threads), printed to stderr when the
// environment sets BLAMM_TIMING.
struct PhaseTiming {
    std::mutex mu;
    double s[6] = {0, 0, 0, 0, 0, 0};
    void add(int k, Clock::duration d)
    {
        std::lock_guard<std::mutex> lk(mu);
        s[k] += std::chrono::duration<double>(d).count();
    }
    void report()
    {
        std::fprintf(stderr, "timing: GPU scan calls %.3f s, ordering hits %.3f s, formatting %.3f s, "
                             "FASTA reading %.3f s (files %.3f s, GPU parsing %.3f s), writing %.3f s\n",
                     s[0], s[1], s[2], s[3] + s[5], s[3], s[5], s[4]);
    }
};
PhaseTiming timing;

// The hits of positions below `payload`, sorted by (position, column): a counting sort
// on position blocks, then small sorts inside each block, blocks split over threads.
std::vector<blamm_hit> orderHits(const std::vector<blamm_hit> &in, int64_t payload, size_t threads)
{
    const int64_t kBlock = 4096;
    const int64_t nb = std::max<int64_t>(1, (payload + kBlock - 1) / kBlock);
    std::vector<int64_t> start((size_t)nb + 1, 0);
    for (const blamm_hit &x : in)
        if (x.pos < payload) ++start[(size_t)(x.pos / kBlock) + 1];
    for (int64_t b = 0; b < nb; ++b) start[(size_t)b + 1] += start[(size_t)b];
    std::vector<blamm_hit> out((size_t)start[(size_t)nb]);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (const blamm_hit &x : in)
        if (x.pos < payload) out[(size_t)fill[(size_t)(x.pos / kBlock)]++] = x;
    const size_t nt = std::max<size_t>(1, std::min<size_t>(threads, out.size() / 100000 + 1));
    auto sortBlocks = [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b)
            std::sort(out.begin() + start[(size_t)b], out.begin() + start[(size_t)b + 1],
                      [](const blamm_hit &a, const blamm_hit &c) { return a.pos != c.pos ? a.pos < c.pos : a.col < c.col; });
    };
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) th.emplace_back(sortBlocks, nb * (int64_t)t / (int64_t)nt, nb * (int64_t)(t + 1) / (int64_t)nt);
    for (auto &x : th) x.join();
    return out;
}

// format "seq\tblamm\tmotif\tstart\tend\tscore\tstrand\t.\t." lines (pwmscan.cpp:88-95);
// floats as the reference's default ostream (%g, 6 significant digits)
void formatHits(const std::vector<blamm_hit> &hits, size_t lo, size_t hi, const StreamChunk &chunk,
                const Species &species, const MotifContainer &motifs, std::string &out)
{
    static const std::string kNone;
    char buf[96];
    for (size_t i = lo; i < hi; ++i) {
        const blamm_hit &h = hits[i];
        const Marker m = chunk.locate(h.pos);
        const Motif &mo = motifs[(size_t)h.col];
        const std::string &seqName =
            (size_t)m.seqIdx < species.seqNames().size() ? species.seqName((size_t)m.seqIdx) : kNone;
        out += seqName;
        out += "\tblamm\t";
        out += mo.name();
        int k = 0;
        buf[k++] = '\t';
        k += formatUnsigned((uint64_t)m.seqPos, buf + k);
        buf[k++] = '\t';
        k += formatUnsigned((uint64_t)(m.seqPos + (int64_t)mo.size()), buf + k);
        buf[k++] = '\t';
        k += formatScore(h.score, buf + k);
        std::memcpy(buf + k, mo.isRevCompl() ? "\t-\t.\t.\n" : "\t+\t.\t.\n", 7);
        out.append(buf, (size_t)k + 7);
    }
}

// A scanned chunk's occurrence lines: its own positions' hits in stream order, formatted
// in parallel slices.  Adds the lines to *nlines.
std::string chunkText(const Device &dev, const StreamChunk &chunk, const Species &sp,
                      const MotifContainer &motifs, size_t numThreads, size_t *nlines)
{
    const auto t1 = Clock::now();
    std::vector<blamm_hit> h = orderHits(dev.hits, chunk.payload, numThreads);
    const auto t2 = Clock::now();
    const size_t nt = std::max<size_t>(1, std::min<size_t>(numThreads, h.size() / 20000 + 1));
    std::vector<std::string> parts(nt);
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t)
        th.emplace_back([&, t] { formatHits(h, h.size() * t / nt, h.size() * (t + 1) / nt, chunk, sp, motifs, parts[t]); });
    for (auto &x : th) x.join();
    std::string text;
    size_t tl = 0;
    for (auto &p : parts) tl += p.size();
    text.reserve(tl);
    for (auto &p : parts) text += p;
    timing.add(1, t2 - t1);
    timing.add(2, Clock::now() - t2);
    *nlines += h.size();
    return text;
}

// One species through the GPU FASTA reader: pieces of its text go to the devices'
// resident streams (blamm_stream_load_fasta), each piece's chunks are scanned in place
// (blamm_scan_stream) and formatted, and the text is written in (piece, chunk) order.
// Returns the occurrences written.
size_t scanSpeciesResident(std::vector<Device> &devs, const Species &sp, const MotifContainer &motifs,
                           const Options &o, std::ostream &os)
{
    const int64_t overlap = (int64_t)motifs.maxMotifLen() - 1;
    const char *env = std::getenv("BLAMM_CHUNK_BASES");
    const int64_t payload = env ? std::max<int64_t>(1, std::atoll(env)) : (int64_t)1 << 26;
    const int64_t maxFilt = (int64_t)sp.totalSeqLength();  // FastaBatch's _maxFiltSeqLen
    FastaPieceReader rd(sp.sequenceFilenames(), ingestPieceBytes());
    struct Out {
        size_t nchunks = SIZE_MAX;
        std::map<size_t, std::string> text;
    };
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::pair<size_t, std::shared_ptr<std::string>>> todo;
    std::map<size_t, Out> done;
    // per piece: its first stream position and sequence index, known once the piece
    // before it is loaded
    std::vector<int64_t> baseStart{0}, seqStart{0};
    size_t nextRead = 0, total = 0;
    bool readerDone = false;
    std::exception_ptr failure;
    std::thread reader([&] {
        try {
            while (true) {
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return todo.size() < devs.size() + 1 || failure; });
                    if (failure) break;
                }
                auto piece = std::make_shared<std::string>();
                const auto t0 = Clock::now();
                const bool more = rd.next(*piece);
                timing.add(3, Clock::now() - t0);
                if (!more) break;
                std::lock_guard<std::mutex> lk(mu);
                todo.emplace_back(nextRead++, std::move(piece));
                cv.notify_all();
            }
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            failure = std::current_exception();
        }
        std::lock_guard<std::mutex> lk(mu);
        readerDone = true;
        cv.notify_all();
    });
    auto worker = [&](Device &dev) {
        try {
            while (true) {
                std::pair<size_t, std::shared_ptr<std::string>> job;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return !todo.empty() || readerDone || failure; });
                    if (failure || (todo.empty() && readerDone)) return;
                    job = todo.front();
                    todo.pop_front();
                    cv.notify_all();
                }
                const size_t p = job.first;
                const auto t0 = Clock::now();
                int64_t nb = 0, nr = 0, ns = 0;
                check(dev.ctx, blamm_stream_load_fasta(dev.ctx, job.second->data(), (int64_t)job.second->size(), &nb,
                                                       &nr, &ns, nullptr),
                      "blamm_stream_load_fasta");
                job.second.reset();
                std::vector<int64_t> rs((size_t)nr), rq((size_t)nr), rp((size_t)nr);
                check(dev.ctx, blamm_stream_tables(dev.ctx, rs.data(), rq.data(), rp.data(), nullptr),
                      "blamm_stream_tables");
                timing.add(5, Clock::now() - t0);
                int64_t b0 = 0, s0 = 0;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return baseStart.size() > p || failure; });
                    if (failure) return;
                    b0 = baseStart[p];
                    s0 = seqStart[p];
                    baseStart.push_back(b0 + nb);
                    seqStart.push_back(s0 + ns);
                    cv.notify_all();
                }
                nb = std::max<int64_t>(0, std::min<int64_t>(nb, maxFilt - b0));
                size_t c = 0;
                for (int64_t begin = 0; begin < nb; begin += payload, ++c) {
                    const int64_t size = std::min<int64_t>(payload + overlap, nb - begin);
                    StreamChunk chunk;
                    residentChunk(rs, rq, rp, begin, size, std::min<int64_t>(payload, size), s0, chunk);
                    const auto t1 = Clock::now();
                    scanChunk(dev, chunk, true, size);
                    timing.add(0, Clock::now() - t1);
                    size_t lines = 0;
                    std::string text = chunkText(dev, chunk, sp, motifs, o.numThreads, &lines);
                    std::lock_guard<std::mutex> lk(mu);
                    total += lines;
                    done[p].text.emplace(c, std::move(text));
                    cv.notify_all();
                }
                std::lock_guard<std::mutex> lk(mu);
                done[p].nchunks = c;
                cv.notify_all();
            }
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            failure = std::current_exception();
            cv.notify_all();
        }
    };
    std::vector<std::thread> workers;
    for (auto &d : devs) workers.emplace_back(worker, std::ref(d));
    // writer (this thread): pieces in order, each piece's chunks in order
    size_t wp = 0, wc = 0;
    while (true) {
        std::string text;
        {
            std::unique_lock<std::mutex> lk(mu);
            bool finished = false;
            cv.wait(lk, [&] {
                if (failure) return true;
                auto it = done.find(wp);
                if (it != done.end() && (it->second.text.count(wc) || it->second.nchunks == wc)) return true;
                finished = readerDone && wp >= nextRead;
                return finished;
            });
            if (failure || finished) break;
            auto it = done.find(wp);
            if (it->second.nchunks == wc) {  // this piece is written out
                done.erase(it);
                ++wp;
                wc = 0;
                continue;
            }
            auto t = it->second.text.find(wc);
            text = std::move(t->second);
            it->second.text.erase(t);
            ++wc;
        }
        const auto t0 = Clock::now();
        os << text;
        timing.add(4, Clock::now() - t0);
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!failure && !(readerDone && wp >= nextRead))
            failure = std::make_exception_ptr(std::runtime_error("writer stopped"));
        cv.notify_all();
    }
    reader.join();
    for (auto &w : workers) w.join();
    if (failure) std::rethrow_exception(failure);
    return total;
}

}  // namespace

// Histogram::generateEmpiricalHist / histThread (hist.cpp:95-160) on the GPU:
// the first maxLength filtered bases of the species, FP32 scores of every
// motif (forward strand) at every position whose window fits its run.
void empiricalHistograms(const Species &species, MotifContainer &motifs, size_t maxLength,
                         std::vector<ScoreHistogram> &hists)
{
    if (motifs.size() == 0) return;
    blamm_ctx *ctx = nullptr;
    if (blamm_ctx_create(0, &ctx) != BLAMM_OK) throw std::runtime_error("cannot create a GPU context");
    std::unique_ptr<blamm_ctx, void (*)(blamm_ctx *)> guard(ctx, blamm_ctx_destroy);
    std::vector<int32_t> lens(motifs.size());
    std::vector<float> thr(motifs.size(), 0.0f), mn(motifs.size()), w(motifs.size());
    for (size_t c = 0; c < motifs.size(); ++c) {
        lens[c] = (int32_t)motifs[c].size();
        mn[c] = hists[c].minScore();
        w[c] = hists[c].width();
    }
    check(ctx, blamm_set_motifs(ctx, motifs.matrix().data(), (int)motifs.matrixRows(), (int)motifs.size(),
                                lens.data(), thr.data()),
          "blamm_set_motifs");
    const size_t nbins = hists[0].numBins();
    std::vector<uint64_t> counts(motifs.size() * nbins, 0);
    if (gpuFastaReader()) {
        // the first maxLength bases of the stream, piece by piece on the device (no window
        // crosses a piece: pieces end where a sequence does)
        FastaPieceReader rd(species.sequenceFilenames(), ingestPieceBytes());
        std::string piece;
        int64_t left = (int64_t)maxLength;
        while (left > 0 && rd.next(piece)) {
            int64_t nb = 0, nr = 0, ns = 0;
            check(ctx, blamm_stream_load_fasta(ctx, piece.data(), (int64_t)piece.size(), &nb, &nr, &ns, nullptr),
                  "blamm_stream_load_fasta");
            std::vector<int64_t> rs((size_t)nr);
            check(ctx, blamm_stream_tables(ctx, rs.data(), nullptr, nullptr, nullptr), "blamm_stream_tables");
            nb = std::min(nb, left);
            left -= nb;
            if (nb == 0) continue;
            std::vector<int64_t> runs;
            for (const int64_t r : rs)
                if (r < nb) runs.push_back(r);
            check(ctx, blamm_score_histograms_stream(ctx, 0, nb, runs.data(), (int64_t)runs.size(), mn.data(),
                                                     w.data(), (int)nbins, counts.data()),
                  "blamm_score_histograms_stream");
        }
    } else {
        FastaStream fs(species.sequenceFilenames(), (int64_t)maxLength);
        StreamChunk chunk;
        const int64_t all = (int64_t)maxLength + 1;
        if (!fs.nextChunk(chunk, all, 0)) return;
        const std::vector<int64_t> runs = chunk.runStarts();
        check(ctx, blamm_score_histograms(ctx, chunk.bases.data(), (int64_t)chunk.bases.size(), runs.data(),
                                          (int64_t)runs.size(), mn.data(), w.data(), (int)nbins, counts.data()),
              "blamm_score_histograms");
    }
    for (size_t c = 0; c < motifs.size(); ++c)
        for (size_t b = 0; b < nbins; ++b) hists[c].counts()[b] += counts[c * nbins + b];
}

int runScanModule(int argc, char **argv)
{
    if (argc < 4) {
        scanUsage();
        exit(EXIT_FAILURE);
    }
    Options o;
    for (int i = 2; i < argc - 2; ++i) {
        const std::string arg(argv[i]);
        if (arg == "-h" || arg == "--help") {
            scanUsage();
            exit(EXIT_SUCCESS);
        } else if (arg == "-rc" || arg == "--revcompl") {
            o.revCompl = true;
        } else if (arg == "-s" || arg == "--simple") {
            o.simple = true;
        } else if (arg == "-c" || arg == "--cuda") {
        } else if ((arg == "-at" || arg == "--absthreshold") && i + 1 < argc - 2) {
            o.absSet = true;
            o.absThreshold = (float)std::atof(argv[++i]);
        } else if ((arg == "-rt" || arg == "--relthreshold") && i + 1 < argc - 2) {
            o.relSet = true;
            o.relThreshold = (float)std::atof(argv[++i]);
            if (o.relThreshold < 0.0 || o.relThreshold > 1.0)
                throw std::runtime_error("The relative threshold should be in range [0..1].");
        } else if ((arg == "-pt" || arg == "--pthreshold") && i + 1 < argc - 2) {
            o.pSet = true;
            o.pvalue = (float)std::atof(argv[++i]);
            if (o.pvalue < 0.0 || o.pvalue > 1.0) throw std::runtime_error("The p-value should be in range [0..1].");
        } else if ((arg == "-t" || arg == "--numthreads") && i + 1 < argc - 2) {
            const int t = std::atoi(argv[++i]);
            if (t < 1) throw std::runtime_error("Number of threads must be a non-zero positive number");
            o.numThreads = (size_t)t;
        } else if ((arg == "-H" || arg == "--histdir") && i + 1 < argc - 2) {
            o.histdir = argv[++i];
            if (o.histdir.back() != '/') o.histdir.push_back('/');
        } else if ((arg == "-o" || arg == "--output") && i + 1 < argc - 2) {
            o.output = argv[++i];
        } else if ((arg == "-m" || arg == "--mode") && i + 1 < argc - 2) {
            const std::string m(argv[++i]);
            if (m == "fp32") o.mode = BLAMM_MODE_FP32;
            else if (m == "bf16") o.mode = BLAMM_MODE_BF16;
            else if (m == "bf16x2") o.mode = BLAMM_MODE_BF16X2;
            else if (m == "auto") o.mode = BLAMM_MODE_AUTO;
            else if (m == "e4m3") o.mode = BLAMM_MODE_E4M3;
            else throw std::runtime_error("unknown mode " + m + " (auto, bf16x2, bf16, e4m3 or fp32)");
        } else {
            scanUsage();
            exit(EXIT_FAILURE);
        }
    }
    if (!(o.absSet || o.relSet || o.pSet)) o.relSet = true;
    if (o.absSet && o.relSet) throw std::runtime_error("Specify either the absolute or relative threshold, not both.");
    if (o.absSet && o.pSet) throw std::runtime_error("Specify either the absolute or p-value threshold, not both.");
    if (o.relSet && o.pSet) throw std::runtime_error("Specify either the relative or p-value threshold, not both.");

    std::cout << "Welcome to blamm -- PWM scan module" << std::endl;
    Settings settings;
    settings.print();
    SpeciesContainer species;
    species.load(std::string(argv[argc - 1]) + ".dict");
    MotifContainer motifs;
    motifs.load(argv[argc - 2], true);
    std::cout << "Loaded " << motifs.size() << " motifs from disk\n";
    std::cout << "Maximum motif size: " << motifs.maxMotifLen() << std::endl;
    if (o.revCompl) {
        motifs.addReverseComplements();
        std::cout << "Scanning both forward and reverse strand of the input sequence(s)" << std::endl;
    } else {
        std::cout << "Scanning only the forward strand of the input sequence(s)" << std::endl;
    }
    motifs.generateMatrixTiles(settings.matrix_P_tile_min_zero_area, true);
    if (o.absSet) std::cout << "Absolute motif score threshold set to: " << o.absThreshold << std::endl;
    else if (o.relSet) std::cout << "Relative motif score threshold set to: " << o.relThreshold << std::endl;
    else std::cout << "P-value motif score threshold set to: " << o.pvalue << std::endl;

    int ndev = 0;
    if (blamm_device_count(&ndev) != BLAMM_OK || ndev == 0) {
        std::cerr << "CUDA error: no devices found. Aborting..." << std::endl;
        return 1;
    }
    if (o.mode != BLAMM_MODE_FP32 && motifs.maxMotifLen() > BLAMM_MAX_TC_MOTIF_LEN) {
        std::cout << "Motifs longer than " << BLAMM_MAX_TC_MOTIF_LEN
                  << " positions: using the plain FP32 GPU scan" << std::endl;
        o.mode = BLAMM_MODE_FP32;
    }
    std::vector<Device> devs((size_t)ndev);
    for (int d = 0; d < ndev; ++d) {
        const int rc = blamm_ctx_create(d, &devs[(size_t)d].ctx);
        if (rc != BLAMM_OK) throw std::runtime_error("cannot create a GPU context on device " + std::to_string(d));
        check(devs[(size_t)d].ctx, blamm_set_mode(devs[(size_t)d].ctx, o.mode), "blamm_set_mode");
        if (o.simple) check(devs[(size_t)d].ctx, blamm_set_softmask(devs[(size_t)d].ctx, 1), "blamm_set_softmask");
    }
    std::cout << "Using " << ndev << " GPU devices" << std::endl;

    std::ofstream ofsCutoff("PWMthresholds.txt");
    std::ofstream os(o.output.c_str(), std::ios::binary);
    if (!os) throw std::runtime_error("Cannot write to file: " + o.output);
    size_t totMatches = 0;

    for (const auto &sp : species) {
        std::cout << "Scanning species: " << sp.name() << std::endl;
        motifs.generateMatrix(sp.nuclCounts(), settings.pseudocount);
        for (auto &m : motifs) {
            if (o.absSet) {
                m.setThreshold(o.absThreshold);
            } else if (o.relSet) {
                const float mx = m.maxScore(), mn = m.minScore();
                m.setThreshold(o.relThreshold * (mx - mn) + mn);
            } else {
                ScoreHistogram h;
                h.loadHistogram(o.histdir, "hist_" + sp.name() + "_" + m.baseName());
                m.setThreshold(h.scoreCutoff(o.pvalue));
            }
        }
        for (auto &m : motifs) {
            if (m.size() > 15) continue;
            ofsCutoff << sp.name() << "\t" << m.name() << "\t" << m.minScore() << "\t" << m.threshold() << "\t"
                      << m.maxScore() << std::endl;
        }
        if (motifs.size() == 0) continue;
        std::vector<int32_t> lens(motifs.size());
        std::vector<float> thr(motifs.size());
        for (size_t c = 0; c < motifs.size(); ++c) {
            lens[c] = (int32_t)motifs[c].size();
            thr[c] = motifs[c].threshold();
        }
        for (auto &d : devs)
            check(d.ctx, blamm_set_motifs(d.ctx, motifs.matrix().data(), (int)motifs.matrixRows(),
                                          (int)motifs.size(), lens.data(), thr.data()),
                  "blamm_set_motifs");

        if (gpuFastaReader()) {
            totMatches += scanSpeciesResident(devs, sp, motifs, o, os);
            std::cout << "Progress... 100%  " << std::endl;
            continue;
        }
        // host reader (BLAMM_FASTA_READER=host) -> per-device workers -> ordered writer
        FastaStream fs(sp.sequenceFilenames(), (int64_t)sp.totalSeqLength());
        const int64_t overlap = (int64_t)motifs.maxMotifLen() - 1;
        const char *env = std::getenv("BLAMM_CHUNK_BASES");
        const int64_t payload = env ? std::max<int64_t>(1, std::atoll(env)) : (int64_t)1 << 26;
        std::mutex mu;
        std::condition_variable cv;
        std::deque<std::pair<size_t, std::shared_ptr<StreamChunk>>> todo;
        std::map<size_t, std::string> done;
        size_t nextRead = 0, nextWrite = 0;
        bool readerDone = false;
        std::exception_ptr failure;
        std::thread reader([&] {
            try {
                while (true) {
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [&] { return todo.size() < devs.size() + 1 || failure; });
                        if (failure) break;
                    }
                    auto chunk = std::make_shared<StreamChunk>();
                    const auto t0 = Clock::now();
                    const bool more = fs.nextChunk(*chunk, payload, overlap);
                    timing.add(3, Clock::now() - t0);
                    if (!more) break;
                    std::lock_guard<std::mutex> lk(mu);
                    todo.emplace_back(nextRead++, chunk);
                    cv.notify_all();
                }
            } catch (...) {
                std::lock_guard<std::mutex> lk(mu);
                failure = std::current_exception();
            }
            std::lock_guard<std::mutex> lk(mu);
            readerDone = true;
            cv.notify_all();
        });
        auto worker = [&](Device &dev) {
            try {
                while (true) {
                    std::pair<size_t, std::shared_ptr<StreamChunk>> job;
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [&] { return !todo.empty() || readerDone || failure; });
                        if (failure || (todo.empty() && readerDone)) return;
                        job = todo.front();
                        todo.pop_front();
                        cv.notify_all();
                    }
                    const StreamChunk &chunk = *job.second;
                    const auto t0 = Clock::now();
                    scanChunk(dev, chunk);
                    timing.add(0, Clock::now() - t0);
                    // the chunk's own positions (the overlap belongs to the next chunk)
                    size_t lines = 0;
                    std::string text = chunkText(dev, chunk, sp, motifs, o.numThreads, &lines);
                    std::unique_lock<std::mutex> lk(mu);
                    totMatches += lines;
                    done.emplace(job.first, std::move(text));
                    cv.notify_all();
                }
            } catch (...) {
                std::lock_guard<std::mutex> lk(mu);
                failure = std::current_exception();
                cv.notify_all();
            }
        };
        std::vector<std::thread> workers;
        for (auto &d : devs) workers.emplace_back(worker, std::ref(d));
        // writer (this thread): chunks in stream order
        while (true) {
            std::string text;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] {
                    return failure || done.count(nextWrite) || (readerDone && todo.empty() && nextWrite >= nextRead &&
                                                                 done.empty());
                });
                if (failure) break;
                auto it = done.find(nextWrite);
                if (it == done.end()) {
                    if (readerDone && todo.empty() && nextWrite >= nextRead) break;
                    continue;
                }
                text = std::move(it->second);
                done.erase(it);
                ++nextWrite;
            }
            const auto t0 = Clock::now();
            os << text;
            timing.add(4, Clock::now() - t0);
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            if (!failure && !readerDone) failure = std::make_exception_ptr(std::runtime_error("writer stopped"));
            cv.notify_all();
        }
        reader.join();
        for (auto &w : workers) w.join();
        if (failure) std::rethrow_exception(failure);
        std::cout << "Progress... 100%  " << std::endl;
    }
    os.close();
    ofsCutoff.close();
    for (auto &d : devs) blamm_ctx_destroy(d.ctx);
    std::cout << "\nWrote " << totMatches << " matches to " << o.output << ".\n";
    if (std::getenv("BLAMM_TIMING")) timing.report();
    return 0;
}

}  // namespace blamm
