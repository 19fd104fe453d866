// hg_fasta.cpp - streaming FASTA in, aligned FASTA out (hg_align_fasta):
// the file edge of the align-to-center path with the reader, the GPU and
// the writer overlapped.
//
// The center FASTA holds one record (aligned to, as the reference CLI's -c)
// or several of one length (multi-reference mode with --keep-length: each
// query is aligned to its best reference, hg_refset_align; the reference
// CLI runs its external MSA over the references first, and its output here
// matches that MSA returning them unchanged).  The output starts with the
// center record(s) through the reference's clean_table.
//
// A reader thread parses the query FASTA into chunks (HAlign-4's
// KseqReader::next, src/utils/seq_io.cpp:134-155: sequence lines joined,
// a trailing '\r' dropped), the calling thread packs each chunk (hg_pack)
// and aligns it with rows (hg_align_batch), and a writer thread writes the
// rows in the reference's output order (mergeAlignedResults with
// --keep-length, src/align/ref_aligner.cpp:676-740): the center record,
// then every row whose CIGAR has an insertion, then every other row, each
// group in input order.  Insertion rows go straight to the output; the
// others go to a side file appended at the end, so nothing is held in
// memory beyond two chunks.
#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/halign_gb300.h"
#include "hg_internal.h"

namespace {

struct Chunk {
    std::vector<std::string> names;
    std::string seqs;
    std::vector<int64_t> offs{0};
    // alignment results
    std::vector<uint8_t> rows, has_ins;
    int64_t stride = 0;
    bool last = false;
};

template <typename T>
class Queue {  // bounded hand-off between two threads
public:
    explicit Queue(size_t cap) : cap_(cap) {}
    void push(T v)
    {
        std::unique_lock<std::mutex> l(mu_);
        not_full_.wait(l, [&] { return q_.size() < cap_; });
        q_.push_back(std::move(v));
        not_empty_.notify_one();
    }
    T pop()
    {
        std::unique_lock<std::mutex> l(mu_);
        not_empty_.wait(l, [&] { return !q_.empty(); });
        T v = std::move(q_.front());
        q_.pop_front();
        not_full_.notify_one();
        return v;
    }

private:
    size_t cap_;
    std::deque<T> q_;
    std::mutex mu_;
    std::condition_variable not_full_, not_empty_;
};

// Record reader with kseq's FASTA conventions: the header's first word is
// the name, the rest the description; sequence lines are joined.
class Reader {
public:
    explicit Reader(const char* path) : f_(path, std::ios::binary) {}
    bool ok() const { return (bool)f_; }
    bool next(std::string& name, std::string& desc, std::string& seq)
    {
        std::string line;
        if (pending_.empty()) {
            while (std::getline(f_, line))
                if (!line.empty() && line[0] == '>') {
                    pending_ = line;
                    break;
                }
            if (pending_.empty()) return false;
        }
        std::string head = pending_.substr(1);
        pending_.clear();
        if (!head.empty() && head.back() == '\r') head.pop_back();
        const size_t sp = head.find_first_of(" \t");
        name = head.substr(0, sp);
        desc = sp == std::string::npos ? std::string() : head.substr(head.find_first_not_of(" \t", sp));
        seq.clear();
        while (std::getline(f_, line)) {
            if (!line.empty() && line[0] == '>') {
                pending_ = line;
                break;
            }
            seq += line;
            if (seq.size() > 1 && seq.back() == '\r') seq.pop_back();
        }
        return true;
    }

private:
    std::ifstream f_;
    std::string pending_;
};

}  // namespace

namespace {

// clean_table (include/utils.h:161-191): A C G T U (either case) and '-'
// kept in upper case, every other byte 'N'; the reference CLI writes the
// center / reference records through it (writeConsensusAndReferences,
// src/align/ref_aligner.cpp:541-556).
std::string cleaned(const std::string& s)
{
    std::string o(s);
    for (char& c : o) {
        switch (c) {
        case 'A': case 'a': c = 'A'; break;
        case 'C': case 'c': c = 'C'; break;
        case 'G': case 'g': c = 'G'; break;
        case 'T': case 't': c = 'T'; break;
        case 'U': case 'u': c = 'U'; break;
        case '-': break;
        default: c = 'N';
        }
    }
    return o;
}

// The streamed run once the center record(s) are known.
int align_stream(const std::vector<std::string>& cnames, const std::vector<std::string>& cdescs,
                 const std::vector<std::string>& cseqs, const char* queries_fasta, const char* out_fasta, int k, int w,
                 int64_t chunk_queries, int64_t* n_aligned)
{
    const bool multi = cseqs.size() > 1;
    const int64_t L = (int64_t)cseqs[0].size();
    for (const auto& s : cseqs)
        if ((int64_t)s.size() != L)
            return hg::set_error(HG_ERR_ARG, "hg_align_fasta: references of different lengths (the reference CLI "
                                             "aligns them with its external MSA tool first)");
    hg_index_t* ix = nullptr;
    hg_refset_t* rs = nullptr;
    int r = HG_OK;
    if (!multi) r = hg_index_create(cseqs[0].data(), L, k, w, nullptr, &ix);
    if (r) return r;
    Reader qr(queries_fasta);
    if (!qr.ok()) {
        hg_index_destroy(ix);
        return hg::set_error(HG_ERR_ARG, "hg_align_fasta: cannot read " + std::string(queries_fasta));
    }
    std::ofstream out(out_fasta, std::ios::binary);
    const std::string rest_path = std::string(out_fasta) + ".rest";
    std::ofstream rest(rest_path, std::ios::binary);
    if (!out || !rest) {
        hg_index_destroy(ix);
        return hg::set_error(HG_ERR_ARG, "hg_align_fasta: cannot write " + std::string(out_fasta));
    }
    for (size_t i = 0; i < cseqs.size(); ++i)
        out << '>' << cnames[i] << (cdescs[i].empty() ? "" : " ") << cdescs[i] << '\n' << cleaned(cseqs[i]) << '\n';
    // reader thread
    Queue<Chunk> in_q(2), out_q(2);
    std::thread reader([&] {
        std::string name, desc, seq;
        for (;;) {
            Chunk c;
            bool more = true;
            while ((int64_t)c.names.size() < chunk_queries && (more = qr.next(name, desc, seq))) {
                c.names.push_back(name);
                c.seqs += seq;
                c.offs.push_back((int64_t)c.seqs.size());
            }
            c.last = !more;
            const bool last = c.last;
            in_q.push(std::move(c));
            if (last) return;
        }
    });
    // writer thread: insertion rows to the output, the others to the side file
    std::thread writer([&] {
        for (;;) {
            Chunk c = out_q.pop();
            for (size_t i = 0; i < c.names.size(); ++i) {
                std::ofstream& o = c.has_ins[i] ? out : rest;
                o.put('>');
                o << c.names[i];
                o.put('\n');
                o.write(reinterpret_cast<const char*>(c.rows.data()) + i * c.stride, (std::streamsize)L);
                o.put('\n');
            }
            if (c.last) return;
        }
    });
    // align chunk by chunk
    hg_ctx_t* ctx = nullptr;
    int64_t ctx_bases = 0;
    int64_t total = 0;
    int rc = HG_OK;
    std::string err;
    for (bool last = false; !last;) {
        Chunk c = in_q.pop();
        last = c.last;
        const int64_t n = (int64_t)c.names.size();
        if (n > 0 && rc == HG_OK) {
            int64_t maxlen = 0;
            for (int64_t i = 0; i < n; ++i) maxlen = std::max(maxlen, c.offs[i + 1] - c.offs[i]);
            // sub-batches of the chunk hold about chunk_queries center-length
            // queries; a longer query than the context holds gets a new one
            if ((!ctx && !rs) || maxlen > ctx_bases) {
                if (ctx) hg_ctx_destroy(ctx), ctx = nullptr;
                if (rs) hg_refset_destroy(rs), rs = nullptr;
                // (at most ~0.9 Gbp per sub-batch: the arenas scale with it)
                ctx_bases = std::max<int64_t>(std::min<int64_t>(chunk_queries * (L + L / 4 + 64), 900000000),
                                              2 * maxlen);
                if (!multi) {
                    rc = hg_ctx_create(ix, chunk_queries, ctx_bases, &ctx);
                } else {  // RefAligner's settings: sketch size 2000, seed 42
                    std::vector<const char*> ptr;
                    std::vector<int64_t> lens;
                    for (const auto& s : cseqs) ptr.push_back(s.data()), lens.push_back((int64_t)s.size());
                    rc = hg_refset_create(ptr.data(), lens.data(), (int)cseqs.size(), k, w, 2000, 42, nullptr,
                                          chunk_queries, ctx_bases, &rs);
                }
            }
            int64_t pb = 0, ne = 0;
            std::vector<uint8_t> packed;
            std::vector<int64_t> poff((size_t)n), eoff((size_t)n + 1);
            std::vector<int32_t> exc, qlen((size_t)n);
            if (rc == HG_OK) rc = hg_pack(c.seqs.data(), c.offs.data(), n, nullptr, 0, nullptr, nullptr, 0, nullptr, &pb, &ne);
            if (rc == HG_OK) {
                packed.resize((size_t)std::max<int64_t>(pb, 16));
                exc.resize((size_t)std::max<int64_t>(ne, 1) * 3);
                rc = hg_pack(c.seqs.data(), c.offs.data(), n, packed.data(), (int64_t)packed.size(), poff.data(),
                             exc.data(), ne, eoff.data(), nullptr, nullptr);
            }
            if (rc == HG_OK) {
                for (int64_t i = 0; i < n; ++i) qlen[i] = (int32_t)(c.offs[i + 1] - c.offs[i]);
                c.stride = (L + 15) / 16 * 16;
                c.rows.resize((size_t)(n * c.stride));
                c.has_ins.resize((size_t)n);
                std::vector<int64_t> coff((size_t)n + 1);
                std::vector<uint32_t> st((size_t)n);
                std::vector<uint32_t> cig((size_t)(c.seqs.size() / 8 + 64 * n + 1024));
                auto run = [&] {
                    return multi ? hg_refset_align(rs, packed.data(), poff.data(), qlen.data(), exc.data(),
                                                   eoff.data(), n, 1, nullptr, nullptr, cig.data(), (int64_t)cig.size(),
                                                   coff.data(), c.has_ins.data(), c.rows.data(), c.stride, st.data())
                                 : hg_align_batch(ctx, packed.data(), poff.data(), qlen.data(), exc.data(),
                                                  eoff.data(), n, cig.data(), (int64_t)cig.size(), coff.data(),
                                                  c.has_ins.data(), c.rows.data(), c.stride, st.data());
                };
                rc = run();
                if (rc == HG_ERR_CAPACITY) {  // CIGARs longer than the first guess: the worst case fits
                    cig.resize((size_t)(c.seqs.size() + n * (L + 4)));
                    rc = run();
                }
            }
            if (rc) err = hg_last_error();
            else total += n;
        }
        if (rc) {  // keep the threads moving; the output is abandoned
            c.names.clear();
        }
        std::string().swap(c.seqs);
        out_q.push(std::move(c));
    }
    reader.join();
    writer.join();
    if (ctx) hg_ctx_destroy(ctx);
    if (rs) hg_refset_destroy(rs);
    hg_index_destroy(ix);
    rest.close();
    if (rc == HG_OK) {  // the rows without insertions follow the insertion rows
        std::ifstream in(rest_path, std::ios::binary);
        if (in.peek() != std::ifstream::traits_type::eof()) out << in.rdbuf();
    }
    out.close();
    std::remove(rest_path.c_str());
    if (rc) return hg::set_error(rc, err);
    if (n_aligned) *n_aligned = total;
    return out ? HG_OK : hg::set_error(HG_ERR_ARG, "hg_align_fasta: write failed");
}

}  // namespace

extern "C" int hg_align_fasta(const char* center_fasta, const char* queries_fasta, const char* out_fasta, int k,
                              int w, int64_t chunk_queries, int64_t* n_aligned)
{
    if (!center_fasta || !queries_fasta || !out_fasta || chunk_queries <= 0)
        return hg::set_error(HG_ERR_ARG, "hg_align_fasta: bad arguments");
    // the center FASTA: one record (align to its consensus) or several
    // (multi-reference mode: each query to its best reference)
    Reader cr(center_fasta);
    std::vector<std::string> cnames, cdescs, cseqs;
    {
        std::string name, desc, seq;
        while (cr.ok() && cr.next(name, desc, seq)) cnames.push_back(name), cdescs.push_back(desc), cseqs.push_back(seq);
    }
    if (cseqs.empty() || cseqs[0].empty())
        return hg::set_error(HG_ERR_ARG, "hg_align_fasta: no center record in " + std::string(center_fasta));
    return align_stream(cnames, cdescs, cseqs, queries_fasta, out_fasta, k, w, chunk_queries, n_aligned);
}

extern "C" int hg_build_center(const char* queries_fasta, int64_t cons_n, char* out, int64_t cap, int64_t* len)
{
    if (!queries_fasta || cons_n <= 0 || !len) return hg::set_error(HG_ERR_ARG, "hg_build_center: bad arguments");
    // preprocessInputFasta's Top-K (src/utils/preprocess.cpp:111-150,
    // TopKLongestSelector, src/consensus/selector.cpp): the cons_n longest
    // records, ties to the earlier record, ordered longest first
    std::vector<std::pair<int64_t, int64_t>> lens;  // (length, input order)
    {
        Reader r(queries_fasta);
        if (!r.ok()) return hg::set_error(HG_ERR_ARG, "hg_build_center: cannot read " + std::string(queries_fasta));
        std::string name, desc, seq;
        for (int64_t i = 0; r.next(name, desc, seq); ++i) lens.emplace_back((int64_t)seq.size(), i);
    }
    if (lens.empty()) return hg::set_error(HG_ERR_ARG, "hg_build_center: no record in " + std::string(queries_fasta));
    auto better = [](const std::pair<int64_t, int64_t>& a, const std::pair<int64_t, int64_t>& b) {
        return a.first != b.first ? a.first > b.first : a.second < b.second;
    };
    const size_t kk = (size_t)std::min<int64_t>(cons_n, (int64_t)lens.size());
    std::partial_sort(lens.begin(), lens.begin() + (long)kk, lens.end(), better);
    lens.resize(kk);
    std::vector<std::pair<int64_t, int64_t>> by_order(lens);
    std::sort(by_order.begin(), by_order.end(), [](auto& a, auto& b) { return a.second < b.second; });
    std::vector<std::string> rows(kk);
    {
        Reader r(queries_fasta);
        std::string name, desc, seq;
        size_t j = 0;
        for (int64_t i = 0; j < kk && r.next(name, desc, seq); ++i) {
            if (i != by_order[j].second) continue;
            const size_t rank = (size_t)(std::lower_bound(lens.begin(), lens.end(), by_order[j], better) - lens.begin());
            rows[rank] = cleaned(seq);  // preprocessing cleans every record
            ++j;
        }
    }
    // the MSA of the selection is the caller's tool; without one the records
    // must already share one length (the CLI with an MSA command that copies)
    for (const auto& s : rows)
        if (s.size() != rows[0].size())
            return hg::set_error(HG_ERR_ARG, "hg_build_center: the selected records differ in length (the reference "
                                             "CLI aligns them with its external MSA tool first)");
    std::string cons;
    const int rc = hg::consensus_of_rows(rows, (size_t)cons_n, cons);
    if (rc) return rc;
    *len = (int64_t)cons.size();
    if ((int64_t)cons.size() > cap || (!out && !cons.empty()))
        return hg::set_error(HG_ERR_CAPACITY, "hg_build_center: cap below the center length");
    std::memcpy(out, cons.data(), cons.size());
    return HG_OK;
}

extern "C" int hg_align_fasta_consensus(const char* queries_fasta, const char* out_fasta, int k, int w, int64_t cons_n,
                                        int64_t chunk_queries, int64_t* n_aligned)
{
    if (!queries_fasta || !out_fasta || chunk_queries <= 0 || cons_n <= 0)
        return hg::set_error(HG_ERR_ARG, "hg_align_fasta_consensus: bad arguments");
    int64_t L = 0;
    int rc = hg_build_center(queries_fasta, cons_n, nullptr, 0, &L);
    if (rc != HG_OK && rc != HG_ERR_CAPACITY) return rc;
    std::string cons((size_t)L, '\0');
    rc = hg_build_center(queries_fasta, cons_n, cons.data(), L, &L);
    if (rc) return rc;
    if (cons.empty()) return hg::set_error(HG_ERR_ARG, "hg_align_fasta_consensus: empty center");
    // the CLI writes the center as ">consensus" (consensus::writeConsensusFasta)
    return align_stream({"consensus"}, {""}, {cons}, queries_fasta, out_fasta, k, w, chunk_queries, n_aligned);
}
