// ingest.cpp -- see ingest.h.
#include "ingest.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace blamm {

bool gpuFastaReader()
{
    const char *e = std::getenv("BLAMM_FASTA_READER");
    return !(e && std::strcmp(e, "host") == 0);
}

size_t ingestPieceBytes()
{
    const char *e = std::getenv("BLAMM_INGEST_PIECE_BYTES");
    const long long v = e ? std::atoll(e) : 0;
    return v > 0 ? (size_t)v : (size_t)256 << 20;
}

FastaPieceReader::FastaPieceReader(std::vector<std::string> files, size_t pieceBytes)
    : files_(std::move(files)), pieceBytes_(std::max<size_t>(pieceBytes, 1))
{
}

bool FastaPieceReader::readMore()
{
    constexpr size_t kRead = size_t(64) << 20;
    while (true) {
        if (ifs_.is_open()) {
            const size_t old = buf_.size();
            buf_.resize(old + kRead);
            ifs_.read(&buf_[old], (std::streamsize)kRead);
            const size_t got = (size_t)ifs_.gcount();
            buf_.resize(old + got);
            if (got > 0) lastNewline_ = buf_.back() == '\n';
            if (got == kRead) return true;
            // end of this file: its last line ends here
            ifs_.close();
            if (!lastNewline_) buf_.push_back('\n');
            lastNewline_ = true;
            if (got > 0) return true;
            continue;
        }
        if (fileIdx_ >= files_.size()) return false;
        ifs_.clear();
        ifs_.open(files_[fileIdx_], std::ios::binary);
        if (!ifs_) throw std::runtime_error("Could not open file: " + files_[fileIdx_]);
        ++fileIdx_;
    }
}

bool FastaPieceReader::next(std::string &piece)
{
    size_t from = pieceBytes_;
    while (true) {
        if (buf_.size() > from) {
            // the first header line that starts at or after pieceBytes_
            const size_t p = buf_.find("\n>", from - 1);
            if (p != std::string::npos) {
                piece.assign(buf_, 0, p + 1);
                buf_.erase(0, p + 1);
                return true;
            }
            from = buf_.size();  // search only the new text next time
        }
        if (!readMore()) {
            if (buf_.empty()) return false;
            piece.swap(buf_);
            buf_.clear();
            return true;
        }
    }
}

std::vector<std::string> headerNames(const std::string &raw, const std::vector<int64_t> &headerPos)
{
    auto space = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; };
    std::vector<std::string> names;
    names.reserve(headerPos.size());
    for (const int64_t h : headerPos) {
        size_t p = (size_t)h + 1;
        while (p < raw.size() && raw[p] != '\n' && space(raw[p])) ++p;
        size_t q = p;
        while (q < raw.size() && raw[q] != '\n' && !space(raw[q])) ++q;
        names.emplace_back(raw, p, q - p);
    }
    return names;
}

void residentChunk(const std::vector<int64_t> &runStart, const std::vector<int64_t> &runSeq,
                   const std::vector<int64_t> &runSeqPos, int64_t begin, int64_t size, int64_t payload,
                   int64_t seqBase, StreamChunk &chunk)
{
    chunk.offset = begin;
    chunk.payload = payload;
    chunk.bases.clear();
    chunk.markers.clear();
    // the run in effect at begin, rebased to chunk position 0, then the runs that start inside
    auto it = std::upper_bound(runStart.begin(), runStart.end(), begin);
    size_t k = (size_t)(it - runStart.begin());
    if (k > 0) {
        const size_t r = k - 1;
        chunk.markers.push_back(Marker{0, seqBase + runSeq[r], runSeqPos[r] + (begin - runStart[r])});
    }
    for (; k < runStart.size() && runStart[k] < begin + size; ++k)
        chunk.markers.push_back(Marker{runStart[k] - begin, seqBase + runSeq[k], runSeqPos[k]});
}

}  // namespace blamm
