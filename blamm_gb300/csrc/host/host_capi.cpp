// host_capi.cpp -- the C ABI of include/blamm_host.h over MotifContainer.
#include <cstring>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "blamm_host.h"
#include "format.h"
#include "histogram.h"
#include "ingest.h"
#include "motif.h"
#include "sequence.h"

struct blamm_bank {
    blamm::MotifContainer motifs;
};

struct blamm_fasta {
    blamm::FastaStream stream;
    blamm::StreamChunk chunk;
    std::vector<int64_t> pos, seq, seqpos;
    explicit blamm_fasta(std::vector<std::string> files, int64_t maxFilt) : stream(std::move(files), maxFilt) {}
};

static thread_local std::string g_err;

template <typename F>
static int guarded(F &&f)
{
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

extern "C" {

const char *blamm_host_last_error(void) { return g_err.c_str(); }

int blamm_bank_load(const char *motif_file, int load_permutations, int revcompl, blamm_bank **out)
{
    if (!motif_file || !out) return -1;
    return guarded([&] {
        auto *b = new blamm_bank();
        try {
            b->motifs.load(motif_file, load_permutations != 0);
            if (revcompl) b->motifs.addReverseComplements();
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int blamm_bank_from_pfms(const uint64_t *pfm, const int32_t *lengths, int nmotifs, int revcompl, blamm_bank **out)
{
    if (!pfm || !lengths || nmotifs < 0 || !out) return -1;
    return guarded([&] {
        // write a Cluster-Buster stream and load it through the same parser/sort
        std::string text;
        size_t k = 0;
        for (int i = 0; i < nmotifs; ++i) {
            text += ">M" + std::to_string(i) + "\n";
            for (int j = 0; j < lengths[i]; ++j, ++k) {
                for (int b = 0; b < 4; ++b) {
                    text += std::to_string(pfm[4 * k + b]);
                    text += b < 3 ? '\t' : '\n';
                }
            }
        }
        char path[] = "/tmp/blamm_bank_XXXXXX";
        const int fd = mkstemp(path);
        if (fd < 0) throw std::runtime_error("cannot create a temporary file");
        FILE *f = fdopen(fd, "w");
        fwrite(text.data(), 1, text.size(), f);
        fclose(f);
        auto *b = new blamm_bank();
        try {
            b->motifs.load(path, true);
            if (revcompl) b->motifs.addReverseComplements();
        } catch (...) {
            remove(path);
            delete b;
            throw;
        }
        remove(path);
        *out = b;
    });
}

void blamm_bank_free(blamm_bank *bank) { delete bank; }

int blamm_bank_columns(const blamm_bank *bank) { return bank ? (int)bank->motifs.size() : -1; }

int blamm_bank_max_len(const blamm_bank *bank) { return bank ? (int)bank->motifs.maxMotifLen() : -1; }

int blamm_bank_generate(blamm_bank *bank, const uint64_t bg_counts[4], float pseudo)
{
    if (!bank || !bg_counts) return -1;
    return guarded([&] {
        bank->motifs.generateMatrix({bg_counts[0], bg_counts[1], bg_counts[2], bg_counts[3]}, pseudo);
    });
}

int blamm_bank_matrix(const blamm_bank *bank, float *P, int32_t *lengths, int32_t *revcompl)
{
    if (!bank) return -1;
    const auto &m = bank->motifs;
    if (P) std::memcpy(P, m.matrix().data(), sizeof(float) * m.matrix().size());
    for (size_t c = 0; c < m.size(); ++c) {
        if (lengths) lengths[c] = (int32_t)m[c].size();
        if (revcompl) revcompl[c] = m[c].isRevCompl() ? 1 : 0;
    }
    return 0;
}

int blamm_bank_min_max(const blamm_bank *bank, float *mn, float *mx)
{
    if (!bank || !mn || !mx) return -1;
    for (size_t c = 0; c < bank->motifs.size(); ++c) {
        mn[c] = bank->motifs[c].minScore();
        mx[c] = bank->motifs[c].maxScore();
    }
    return 0;
}

int blamm_bank_pvalue_thresholds(const blamm_bank *bank, const float bg_prob[4], int nbins, uint64_t max_length,
                                 float pvalue, float *thr)
{
    if (!bank || !bg_prob || nbins < 2 || !thr) return -1;
    return guarded([&] {
        const std::array<float, 4> bg{bg_prob[0], bg_prob[1], bg_prob[2], bg_prob[3]};
        std::map<std::string, float> cache;  // base name -> threshold of its forward motif
        for (size_t c = 0; c < bank->motifs.size(); ++c) {
            const blamm::Motif &m = bank->motifs[c];
            if (m.isRevCompl()) continue;
            const std::string key = m.baseName();
            if (cache.count(key)) continue;
            blamm::ScoreHistogram h(m.minScore(), m.maxScore(), (size_t)nbins);
            blamm::theoreticalHistogram(m, bg, (size_t)max_length, h);
            cache[key] = h.scoreCutoff(pvalue);
        }
        for (size_t c = 0; c < bank->motifs.size(); ++c) {
            const std::string key = bank->motifs[c].baseName();
            auto it = cache.find(key);
            if (it == cache.end()) throw std::runtime_error("no forward motif for " + key);
            thr[c] = it->second;
        }
    });
}

int blamm_bank_hist_columns(const blamm_bank *bank, int32_t *hist_of)
{
    if (!bank || !hist_of) return -1;
    return guarded([&] {
        std::map<std::string, int32_t> fwd;  // base name -> first forward column
        for (size_t c = 0; c < bank->motifs.size(); ++c) {
            const blamm::Motif &m = bank->motifs[c];
            if (!m.isRevCompl() && !fwd.count(m.baseName())) fwd[m.baseName()] = (int32_t)c;
        }
        for (size_t c = 0; c < bank->motifs.size(); ++c) {
            auto it = fwd.find(bank->motifs[c].baseName());
            if (it == fwd.end()) throw std::runtime_error("no forward motif for " + bank->motifs[c].baseName());
            hist_of[c] = it->second;
        }
    });
}

int blamm_format_scores(const float *values, int64_t n, char *out, int stride)
{
    if ((n > 0 && (!values || !out)) || n < 0 || stride < 16) return -1;
    for (int64_t i = 0; i < n; ++i) blamm::formatScore(values[i], out + i * stride);
    return 0;
}

const char *blamm_bank_name(const blamm_bank *bank, int c)
{
    if (!bank || c < 0 || (size_t)c >= bank->motifs.size()) return nullptr;
    return bank->motifs[(size_t)c].name().c_str();
}

int blamm_fasta_open(const char *const *files, int nfiles, int64_t max_filt, blamm_fasta **out)
{
    if (!files || nfiles < 0 || !out) return -1;
    return guarded([&] {
        std::vector<std::string> v(files, files + nfiles);
        *out = new blamm_fasta(v, max_filt < 0 ? std::numeric_limits<int64_t>::max() : max_filt);
    });
}

int blamm_fasta_next(blamm_fasta *f, int64_t payload, int64_t overlap, const char **bases, int64_t *size,
                     int64_t *chunk_payload, int64_t *offset, const int64_t **marker_pos,
                     const int64_t **marker_seq, const int64_t **marker_seqpos, int64_t *nmarkers)
{
    if (!f || payload <= 0 || overlap < 0) return -1;
    int got = 0;
    const int rc = guarded([&] {
        got = f->stream.nextChunk(f->chunk, payload, overlap) ? 1 : 0;
        if (!got) return;
        f->pos.clear();
        f->seq.clear();
        f->seqpos.clear();
        for (const auto &m : f->chunk.markers) {
            f->pos.push_back(m.streamPos);
            f->seq.push_back(m.seqIdx);
            f->seqpos.push_back(m.seqPos);
        }
        if (bases) *bases = f->chunk.bases.data();
        if (size) *size = (int64_t)f->chunk.bases.size();
        if (chunk_payload) *chunk_payload = f->chunk.payload;
        if (offset) *offset = f->chunk.offset;
        if (marker_pos) *marker_pos = f->pos.data();
        if (marker_seq) *marker_seq = f->seq.data();
        if (marker_seqpos) *marker_seqpos = f->seqpos.data();
        if (nmarkers) *nmarkers = (int64_t)f->pos.size();
    });
    return rc ? rc : got;
}

int64_t blamm_fasta_num_sequences(const blamm_fasta *f) { return f ? (int64_t)f->stream.seqNames().size() : -1; }

const char *blamm_fasta_sequence_name(const blamm_fasta *f, int64_t i)
{
    if (!f || i < 0 || (size_t)i >= f->stream.seqNames().size()) return nullptr;
    return f->stream.seqNames()[(size_t)i].c_str();
}

void blamm_fasta_close(blamm_fasta *f) { delete f; }

struct blamm_fasta_pieces {
    blamm::FastaPieceReader reader;
    std::string piece;
    blamm_fasta_pieces(std::vector<std::string> files, size_t bytes) : reader(std::move(files), bytes) {}
};

int blamm_fasta_pieces_open(const char *const *files, int nfiles, int64_t piece_bytes, blamm_fasta_pieces **out)
{
    if (!files || nfiles < 0 || piece_bytes <= 0 || !out) return -1;
    return guarded([&] {
        std::vector<std::string> v(files, files + nfiles);
        *out = new blamm_fasta_pieces(v, (size_t)piece_bytes);
    });
}

int blamm_fasta_pieces_next(blamm_fasta_pieces *p, const char **text, int64_t *size)
{
    if (!p || !text || !size) return -1;
    int got = 0;
    const int rc = guarded([&] { got = p->reader.next(p->piece) ? 1 : 0; });
    if (rc < 0) return rc;
    *text = got ? p->piece.data() : nullptr;
    *size = got ? (int64_t)p->piece.size() : 0;
    return got;
}

void blamm_fasta_pieces_close(blamm_fasta_pieces *p) { delete p; }

int blamm_fasta_header_name(const char *text, int64_t size, int64_t header_pos, char *out, int cap)
{
    if (!text || size < 0 || header_pos < 0 || header_pos >= size || !out || cap <= 0) return -1;
    const std::string t(text, (size_t)size);
    const std::string name = blamm::headerNames(t, {header_pos})[0];
    if ((int64_t)name.size() + 1 > cap) return -1;
    std::memcpy(out, name.data(), name.size());
    out[name.size()] = 0;
    return (int)name.size();
}

}  // extern "C"
