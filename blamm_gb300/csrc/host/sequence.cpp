// sequence.cpp -- see sequence.h.
#include "sequence.h"

#include <algorithm>
#include <sstream>
#include <stdexcept>

namespace blamm {

static inline bool validBase(char c)
{
    switch (c) {
    case 'A': case 'a': case 'C': case 'c': case 'G': case 'g': case 'T': case 't':
        return true;
    default:
        return false;
    }
}

std::vector<int64_t> StreamChunk::runStarts() const
{
    std::vector<int64_t> r;
    r.reserve(markers.size());
    for (const auto &m : markers) r.push_back(m.streamPos);
    return r;
}

Marker StreamChunk::locate(int64_t chunkPos) const
{
    auto it = std::upper_bound(markers.begin(), markers.end(), chunkPos,
                               [](int64_t p, const Marker &m) { return p < m.streamPos; });
    --it;  // last marker <= chunkPos
    return Marker{chunkPos, it->seqIdx, it->seqPos + (chunkPos - it->streamPos)};
}

FastaStream::FastaStream(std::vector<std::string> files, int64_t maxFiltLen)
    : files_(std::move(files)), maxFilt_(maxFiltLen)
{
}

bool FastaStream::readLine(std::string &line)
{
    // FastaBatch::getNextLine / moveToNextFile (sequence.cpp:123-179)
    while (true) {
        if (ifs_.is_open() && std::getline(ifs_, line)) return true;
        if (ifs_.is_open()) ifs_.close();
        if (fileIdx_ >= files_.size()) return false;
        ifs_.clear();
        ifs_.open(files_[fileIdx_]);
        if (!ifs_) throw std::runtime_error("Could not open file: " + files_[fileIdx_]);
        ++fileIdx_;
    }
}

void FastaStream::append(const char *data, int64_t len, int64_t seq, int64_t seqPos)
{
    len = std::min<int64_t>(len, maxFilt_ - filtTotal_);  // FastaBatch::appendNextBlock limit
    if (len <= 0) return;
    const int64_t pos = pendOff_ + (int64_t)pending_.size();
    // SeqBlock::isContiguous (sequence.cpp:35-50)
    const bool contiguous = last_.seqIdx == seq && pos - last_.streamPos == seqPos - last_.seqPos;
    if (!contiguous) {
        last_ = Marker{pos, seq, seqPos};
        pendMarkers_.push_back(last_);
    }
    pending_.append(data, (size_t)len);
    filtTotal_ += len;
}

bool FastaStream::fill(int64_t want)
{
    std::string line;
    while ((int64_t)pending_.size() < want && !eof_) {
        if (filtTotal_ >= maxFilt_ || !readLine(line)) {
            eof_ = true;
            break;
        }
        if (line.empty()) continue;
        if (line[0] == '>') {
            std::istringstream iss(line.substr(1));
            std::string name;
            iss >> name;
            names_.push_back(name);
            curSeqLen_ = 0;
            continue;
        }
        if (names_.empty()) throw std::runtime_error("Input file does not appear to be in fasta format\n");
        const int64_t seq = (int64_t)names_.size() - 1, pos0 = curSeqLen_;
        const int64_t len = (int64_t)line.size();
        curSeqLen_ += len;
        totSeqLen_ += len;
        // FastaBatch::filterLine (sequence.cpp:181-214)
        int64_t i = 0;
        while (i < len) {
            while (i < len && !validBase(line[i])) ++i;
            int64_t j = i;
            while (j < len && validBase(line[j])) ++j;
            if (j > i) append(line.data() + i, j - i, seq, pos0 + i);
            i = j;
        }
    }
    return !pending_.empty();
}

bool FastaStream::nextChunk(StreamChunk &chunk, int64_t payload, int64_t overlap)
{
    if (!fill(payload + overlap)) return false;
    const int64_t size = std::min<int64_t>((int64_t)pending_.size(), payload + overlap);
    const int64_t pay = std::min<int64_t>(payload, size);
    chunk.offset = pendOff_;
    chunk.payload = pay;
    chunk.bases.assign(pending_, 0, (size_t)size);
    chunk.markers.clear();
    // first marker: the one in effect at the chunk start, rebased to 0
    size_t k = 0;
    while (k + 1 < pendMarkers_.size() && pendMarkers_[k + 1].streamPos <= pendOff_) ++k;
    const Marker &m0 = pendMarkers_[k];
    chunk.markers.push_back(Marker{0, m0.seqIdx, m0.seqPos + (pendOff_ - m0.streamPos)});
    for (size_t i = k + 1; i < pendMarkers_.size() && pendMarkers_[i].streamPos < pendOff_ + size; ++i)
        chunk.markers.push_back(
            Marker{pendMarkers_[i].streamPos - pendOff_, pendMarkers_[i].seqIdx, pendMarkers_[i].seqPos});
    // consume the payload; keep the marker in effect at the new start
    pending_.erase(0, (size_t)pay);
    pendOff_ += pay;
    size_t keep = 0;
    while (keep + 1 < pendMarkers_.size() && pendMarkers_[keep + 1].streamPos <= pendOff_) ++keep;
    pendMarkers_.erase(pendMarkers_.begin(), pendMarkers_.begin() + (long)keep);
    return true;
}

}  // namespace blamm
