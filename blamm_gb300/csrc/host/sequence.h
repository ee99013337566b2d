// sequence.h -- FASTA streaming into the filtered base stream the GPU scans.
//
// Same semantics as biointec/blamm's FastaBatch / SeqBlock (src/sequence.h,
// src/sequence.cpp:35-293): files are read line by line; '>' lines name a new
// sequence (first whitespace token); sequence lines are split at every
// character outside ACGTacgt; the valid runs are concatenated into one stream
// with a marker wherever the stream stops being contiguous with the sequence
// (new sequence or skipped characters).  The stream is cut into chunks of a
// fixed payload that carry an overlap of (longest motif - 1) bases, like the
// reference's overlapping blocks, but tens of megabases long.
#pragma once

#include <cstdint>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

namespace blamm {

struct Marker {
    int64_t streamPos;  // position in the filtered stream
    int64_t seqIdx;     // sequence index (reading order)
    int64_t seqPos;     // 0-based position of streamPos inside that sequence
};

// A chunk of the filtered stream: bases [0, size) of which [0, payload) are
// this chunk's positions and the rest is the overlap into the next chunk.
struct StreamChunk {
    int64_t offset = 0;   // stream position of chunk base 0
    int64_t payload = 0;  // positions scanned from this chunk
    std::string bases;
    std::vector<Marker> markers;  // markers[0].streamPos == offset (chunk-relative 0)

    // stream-relative start of each run inside the chunk (chunk coordinates)
    std::vector<int64_t> runStarts() const;
    // SeqBlock::getSeqPos (sequence.cpp:52-66) for a chunk position
    Marker locate(int64_t chunkPos) const;
};

class FastaStream {
public:
    // maxFiltLen truncates the stream like FastaBatch's _maxFiltSeqLen
    explicit FastaStream(std::vector<std::string> files,
                         int64_t maxFiltLen = std::numeric_limits<int64_t>::max());

    // Next chunk with `payload` positions and `overlap` extra bases (the
    // overlap is re-used as the start of the following chunk).  Returns false
    // at the end of the stream.
    bool nextChunk(StreamChunk &chunk, int64_t payload, int64_t overlap);

    const std::vector<std::string> &seqNames() const { return names_; }
    int64_t filteredLength() const { return filtTotal_; }
    int64_t totalSeqLength() const { return totSeqLen_; }

private:
    bool readLine(std::string &line);
    bool fill(int64_t want);  // grow pending_ to at least `want` bases (or EOF)
    void append(const char *data, int64_t len, int64_t seq, int64_t seqPos);

    std::vector<std::string> files_;
    size_t fileIdx_ = 0;
    std::ifstream ifs_;
    std::vector<std::string> names_;
    int64_t curSeqLen_ = 0, totSeqLen_ = 0;
    int64_t maxFilt_, filtTotal_ = 0;
    bool eof_ = false;

    // pending stream data not yet handed out: starts at stream position pendOff_
    std::string pending_;
    std::vector<Marker> pendMarkers_;  // absolute stream positions
    int64_t pendOff_ = 0;
    Marker last_{-1, -1, -1};
};

}  // namespace blamm
