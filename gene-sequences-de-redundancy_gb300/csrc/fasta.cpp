// fasta.cpp -- host side of the drop-in boundary: option parsing, FASTA
// reading with the reference's line rules and sort, and the output writer.
//
//   gsdr_check_option  <- checkOption (cuda-version/func.cu:10-92)
//   gsdr_fasta_read    <- readFile    (cuda-version/func.cu:94-117)
//   gsdr_fasta_write   <- saveFile    (cuda-version/func.cu:1099-1111)
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "gsdr.h"
#include "gsdr_host.h"
#include "stdsort.h"

struct gsdr_fasta {
    std::vector<char> buf;          // file bytes, then concatenated multi-line records
    std::vector<int64_t> name_off;  // file order
    std::vector<int64_t> name_len;
    std::vector<int64_t> data_off;  // file order
    std::vector<int32_t> data_len;
    std::vector<int32_t> order;     // sorted position -> file position
    std::vector<int64_t> s_off;     // sorted views for gsdr_reads
    std::vector<int32_t> s_len;
};

namespace {

// Record boundaries follow std::getline over '\n' (func.cu:97-109): the first
// line is a name whatever it holds; later lines starting with '>' open a new
// record; all other lines are appended verbatim (a '\r' stays in the data).
int parse_into(gsdr_fasta* f) {
    const char* b = f->buf.data();
    const int64_t n = (int64_t)f->buf.size();
    struct Span {
        int64_t off, len;
    };
    std::vector<Span> pieces;  // data lines of the current record
    int64_t cur_name_off = 0, cur_name_len = 0;
    std::vector<char> extra;   // concatenations, appended to buf at the end
    std::vector<std::pair<int, int64_t>> extra_fix;  // (record, offset in extra)

    auto finish = [&]() {
        f->name_off.push_back(cur_name_off);
        f->name_len.push_back(cur_name_len);
        int64_t total = 0;
        for (const Span& s : pieces) total += s.len;
        if (total > INT32_MAX) return false;
        if (pieces.size() == 1) {
            f->data_off.push_back(pieces[0].off);
        } else if (pieces.empty()) {
            f->data_off.push_back(0);
        } else {
            extra_fix.emplace_back((int)f->data_off.size(), (int64_t)extra.size());
            f->data_off.push_back(0);
            for (const Span& s : pieces) extra.insert(extra.end(), b + s.off, b + s.off + s.len);
        }
        f->data_len.push_back((int32_t)total);
        pieces.clear();
        return true;
    };

    int64_t pos = 0;
    bool first = true;
    // A file with no bytes still yields one empty record, as in the reference.
    while (true) {
        if (pos >= n) {
            if (first) {
                cur_name_off = 0;
                cur_name_len = 0;
            }
            break;
        }
        const char* nl = (const char*)std::memchr(b + pos, '\n', (size_t)(n - pos));
        int64_t end = nl ? (int64_t)(nl - b) : n;
        int64_t len = end - pos;
        if (first) {
            cur_name_off = pos;
            cur_name_len = len;
            first = false;
        } else if (len > 0 && b[pos] == '>') {
            if (!finish()) return GSDR_EUNSUPPORTED;
            cur_name_off = pos;
            cur_name_len = len;
        } else if (len > 0) {
            pieces.push_back({pos, len});
        }
        pos = end + 1;
        if (!nl) break;
    }
    if (!finish()) return GSDR_EUNSUPPORTED;
    if (!extra.empty()) {
        int64_t base = (int64_t)f->buf.size();
        f->buf.insert(f->buf.end(), extra.begin(), extra.end());
        for (auto& fx : extra_fix) f->data_off[fx.first] = base + fx.second;
    }
    const int32_t count = (int32_t)f->data_len.size();
    f->order.resize(count);
    std::iota(f->order.begin(), f->order.end(), 0);
    // Same call as func.cu:111-113 (std::sort, length descending).  The
    // permutation depends only on the comparison outcomes, so sorting indices
    // reproduces the reference's order of equal-length reads; large inputs
    // run the same sort's independent parts on several threads (stdsort.h).
    const int32_t* dl = f->data_len.data();
    f->s_off.resize(count);
    f->s_len.resize(count);
    // offsets and lengths in sorted order, gathered by the sort's own threads
    const int32_t* ord = f->order.data();
    const int64_t* doff = f->data_off.data();
    int64_t* soff = f->s_off.data();
    int32_t* slen = f->s_len.data();
    const std::function<void(int, int)> gather = [=](int t, int T) {
        const int32_t lo = (int32_t)((int64_t)count * t / T);
        const int32_t hi = (int32_t)((int64_t)count * (t + 1) / T);
        for (int32_t i = lo; i < hi; i++) {
            soff[i] = doff[ord[i]];
            slen[i] = dl[ord[i]];
        }
    };
    gsdr::std_sort_threaded(f->order.begin(), f->order.end(),
                            [dl](const int32_t& a, const int32_t& c) { return dl[a] > dl[c]; },
                            gsdr::sort_threads(), gather);
    return GSDR_OK;
}

}  // namespace

extern "C" {

int gsdr_fasta_parse(const char* data, int64_t n, gsdr_fasta** out) {
    *out = nullptr;
    if (n < 0 || (n > 0 && !data)) return gsdr::fail(GSDR_EINVAL, "fasta: bad buffer");
    gsdr_fasta* f = new (std::nothrow) gsdr_fasta();
    if (!f) return gsdr::fail(GSDR_ENOMEM, "fasta: out of host memory");
    try {
        f->buf.assign(data, data + n);
        int rc = parse_into(f);
        if (rc) {
            delete f;
            return gsdr::fail(rc, "fasta: a record is longer than 2^31-1 bytes");
        }
    } catch (const std::bad_alloc&) {
        delete f;
        return gsdr::fail(GSDR_ENOMEM, "fasta: out of host memory");
    }
    *out = f;
    return GSDR_OK;
}

int gsdr_fasta_read(const char* path, gsdr_fasta** out) {
    *out = nullptr;
    gsdr_fasta* f = new (std::nothrow) gsdr_fasta();
    if (!f) return gsdr::fail(GSDR_ENOMEM, "fasta: out of host memory");
    try {
        FILE* fp = path ? std::fopen(path, "rb") : nullptr;
        if (fp) {  // an unreadable file reads as empty (std::ifstream in func.cu:95)
            std::fseek(fp, 0, SEEK_END);
            long sz = std::ftell(fp);
            std::fseek(fp, 0, SEEK_SET);
            if (sz > 0) {
                f->buf.resize((size_t)sz);
                size_t got = std::fread(f->buf.data(), 1, (size_t)sz, fp);
                f->buf.resize(got);
            }
            std::fclose(fp);
        }
        int rc = parse_into(f);
        if (rc) {
            delete f;
            return gsdr::fail(rc, "fasta: a record is longer than 2^31-1 bytes");
        }
    } catch (const std::bad_alloc&) {
        delete f;
        return gsdr::fail(GSDR_ENOMEM, "fasta: out of host memory");
    }
    *out = f;
    return GSDR_OK;
}

int32_t gsdr_fasta_count(const gsdr_fasta* f) { return f ? (int32_t)f->order.size() : 0; }

int gsdr_fasta_view(const gsdr_fasta* f, gsdr_reads* v) {
    if (!f || !v) return GSDR_EINVAL;
    v->bytes = f->buf.data();
    v->n_bytes = (int64_t)f->buf.size();
    v->offset = f->s_off.data();
    v->length = f->s_len.data();
    v->n = (int32_t)f->order.size();
    return GSDR_OK;
}

const int32_t* gsdr_fasta_order(const gsdr_fasta* f) { return f ? f->order.data() : nullptr; }

const char* gsdr_fasta_name(const gsdr_fasta* f, int32_t i, int64_t* len) {
    if (!f || i < 0 || i >= (int32_t)f->order.size()) return nullptr;
    int32_t r = f->order[i];
    if (len) *len = f->name_len[r];
    return f->buf.data() + f->name_off[r];
}

int gsdr_fasta_format(const gsdr_fasta* f, const int32_t* cluster, char* buf, int64_t cap,
                      int64_t* need) {
    if (!f || !cluster) return GSDR_EINVAL;
    int64_t total = 0;
    const int32_t n = (int32_t)f->order.size();
    for (int32_t i = 0; i < n; i++)
        if (cluster[i] == i) total += f->name_len[f->order[i]] + f->data_len[f->order[i]] + 2;
    if (need) *need = total;
    if (!buf) return GSDR_OK;
    if (cap < total) return GSDR_EINVAL;
    char* p = buf;
    const char* b = f->buf.data();
    for (int32_t i = 0; i < n; i++) {
        if (cluster[i] != i) continue;
        int32_t r = f->order[i];
        std::memcpy(p, b + f->name_off[r], (size_t)f->name_len[r]);
        p += f->name_len[r];
        *p++ = '\n';
        std::memcpy(p, b + f->data_off[r], (size_t)f->data_len[r]);
        p += f->data_len[r];
        *p++ = '\n';
    }
    return GSDR_OK;
}

// Cluster membership as text (no counterpart in the reference, which keeps
// cluster[] in memory): clusters numbered in output order, members in sorted
// order, the representative first and marked '*'.
static int clusters_text(const gsdr_fasta* f, const int32_t* cluster, std::vector<char>& out,
                         int64_t* n_clusters) {
    const int32_t n = (int32_t)f->order.size();
    std::vector<int32_t> cid(n, -1), start(n + 1, 0), member(n);
    int32_t k = 0;
    for (int32_t i = 0; i < n; i++) {
        const int32_t c = cluster[i];
        if (c < 0 || c > i || cluster[c] != c)
            return gsdr::fail(GSDR_EINVAL, "cluster array: not a finished clustering");
        if (c == i) cid[i] = k++;
    }
    for (int32_t i = 0; i < n; i++) start[cid[cluster[i]] + 1]++;
    for (int32_t c = 0; c < k; c++) start[c + 1] += start[c];
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (int32_t i = 0; i < n; i++) member[fill[cid[cluster[i]]]++] = i;
    const char* b = f->buf.data();
    char num[64];
    for (int32_t c = 0; c < k; c++) {
        int len = std::snprintf(num, sizeof(num), ">Cluster %d\n", c);
        out.insert(out.end(), num, num + len);
        for (int32_t m = start[c]; m < start[c + 1]; m++) {
            const int32_t i = member[m];
            const int32_t r = f->order[i];
            len = std::snprintf(num, sizeof(num), "%d\t%lldnt, ", m - start[c],
                                (long long)f->data_len[r]);
            out.insert(out.end(), num, num + len);
            out.insert(out.end(), b + f->name_off[r], b + f->name_off[r] + f->name_len[r]);
            const char* tail = cluster[i] == i ? "... *\n" : "...\n";
            out.insert(out.end(), tail, tail + std::strlen(tail));
        }
    }
    if (n_clusters) *n_clusters = k;
    return GSDR_OK;
}

int gsdr_fasta_format_clusters(const gsdr_fasta* f, const int32_t* cluster, char* buf,
                               int64_t cap, int64_t* need) {
    if (!f || !cluster) return gsdr::fail(GSDR_EINVAL, "null argument");
    std::vector<char> out;
    const int rc = clusters_text(f, cluster, out, nullptr);
    if (rc) return rc;
    if (need) *need = (int64_t)out.size();
    if (!buf) return GSDR_OK;
    if (cap < (int64_t)out.size()) return gsdr::fail(GSDR_EINVAL, "buffer too small");
    std::memcpy(buf, out.data(), out.size());
    return GSDR_OK;
}

int gsdr_fasta_write_clusters(const char* path, const gsdr_fasta* f, const int32_t* cluster,
                              int64_t* n_clusters) {
    if (!f || !cluster || !path) return gsdr::fail(GSDR_EINVAL, "null argument");
    std::vector<char> out;
    const int rc = clusters_text(f, cluster, out, n_clusters);
    if (rc) return rc;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return gsdr::fail(GSDR_EIO, "cannot open cluster file");
    const bool ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
    if (std::fclose(fp) != 0 || !ok) return gsdr::fail(GSDR_EIO, "cannot write cluster file");
    return GSDR_OK;
}

int gsdr_fasta_write(const char* path, const gsdr_fasta* f, const int32_t* cluster,
                     int64_t* n_written) {
    if (!f || !cluster || !path) return GSDR_EINVAL;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return gsdr::fail(GSDR_EIO, "cannot open output file");
    std::vector<char> out;
    out.reserve(1 << 22);
    int64_t count = 0;
    const int32_t n = (int32_t)f->order.size();
    const char* b = f->buf.data();
    bool ok = true;
    for (int32_t i = 0; i < n; i++) {
        if (cluster[i] != i) continue;
        int32_t r = f->order[i];
        out.insert(out.end(), b + f->name_off[r], b + f->name_off[r] + f->name_len[r]);
        out.push_back('\n');
        out.insert(out.end(), b + f->data_off[r], b + f->data_off[r] + f->data_len[r]);
        out.push_back('\n');
        count++;
        if (out.size() >= (1u << 22)) {
            ok = ok && std::fwrite(out.data(), 1, out.size(), fp) == out.size();
            out.clear();
        }
    }
    if (!out.empty()) ok = ok && std::fwrite(out.data(), 1, out.size(), fp) == out.size();
    ok = (std::fclose(fp) == 0) && ok;
    if (n_written) *n_written = count;
    return ok ? GSDR_OK : gsdr::fail(GSDR_EIO, "short write on output file");
}

void gsdr_fasta_free(gsdr_fasta* f) { delete f; }

void gsdr_default_opts(gsdr_opts* o) {
    std::memset(o, 0, sizeof(*o));
    o->threshold = 0.95f;
    o->word_length = 0;
    o->drop = 3;
    o->pigeon = 0;
    o->batch = 0;
    o->device = 0;
}

// The derivations of checkOption (func.cu:43-84).  The float threshold is
// compared with double literals, as C++ does there: 0.88f < 0.88 for example,
// so t = 0.88 gives k = 4.
int gsdr_resolve_opts(gsdr_opts* o, const char** msg) {
    const char* m = nullptr;
    if (!(o->threshold >= 0.8 && o->threshold < 1)) {
        m = "threshold out of range (0.8<=threshold<1)";
    } else if (o->word_length != 0 && (o->word_length < 4 || o->word_length > 12)) {
        m = "word length out of range (4<=word length<=12)";
    } else if (o->drop != 0 && o->drop != 1 && o->drop != 3) {
        m = "drop error (drop=0/1)";
    } else if (o->pigeon != 0 && o->pigeon != 1) {
        m = "pigeon error (pigeon=0/1)";
    } else if (o->batch < 0) {
        m = "batch must be >= 0";
    } else if (o->word_filter < 0 || o->word_filter > 4) {
        m = "word filter form must be 0..4";
    } else if (o->variant != 0 && o->variant != 1) {
        m = "variant must be 0 (cuda-version) or 1 (SYCL program)";
    } else if (o->band_serial < -1) {
        m = "band_serial must be -1, 0 or positive";
    } else if (o->group_words < -1 || o->group_words > 128) {
        m = "group_words must be -1..128";
    } else if (o->align_blocks < 0 || o->align_blocks > 8 || o->filter_blocks < 0 ||
               o->filter_blocks > 8) {
        m = "align_blocks and filter_blocks must be 0..8";
    } else if (o->graph_steps < 0 || o->graph_steps > 64 || (o->graph_steps & 1)) {
        m = "graph_steps must be 0 or even, 2..64";
    } else if (o->variant == 1 && o->word_length != 0 &&
               (o->word_length < 4 || o->word_length > 8)) {
        m = "word length out of range (4<=word length<=8)";  // func.cpp:47-51
    } else if (o->variant == 1 && (o->drop == 1 || o->pigeon != 0)) {
        m = "the SYCL program has no drop mode and no pigeon filter";
    }
    if (m) {
        if (msg) *msg = m;
        return gsdr::fail(GSDR_EINVAL, m);
    }
    if (o->variant == 1) {
        // func.cpp:36-45: the word length rises with t; filters always on
        if (o->word_length == 0) {
            if (o->threshold < 0.88) o->word_length = 4;
            else if (o->threshold < 0.94) o->word_length = 5;
            else if (o->threshold < 0.97) o->word_length = 6;
            else o->word_length = 7;
        }
        o->drop = 0;
        return GSDR_OK;
    }
    if (o->word_length == 0) {
        if (o->threshold < 0.88) o->word_length = 4;
        else if (o->threshold < 0.94) o->word_length = 7;
        else if (o->threshold < 0.97) o->word_length = 6;
        else o->word_length = 5;
    }
    if (o->drop == 3) o->drop = (o->threshold <= 0.879) ? 1 : 0;
    return GSDR_OK;
}

int gsdr_check_option(int argc, char** argv, gsdr_opts* o, char* in_path, char* out_path,
                      int64_t cap) {
    if (!o || !in_path || !out_path || cap < 2) return GSDR_EINVAL;
    gsdr_default_opts(o);
    std::string in = "testData.fasta", out = "result.fasta";
    if (argc % 2 != 1) return gsdr::fail(GSDR_EINVAL, "odd number of option words");
    bool drop_key = false, pigeon_key = false;
    for (int i = 1; i < argc; i += 2) {
        const char* key = argv[i];
        while (*key == '-') key++;  // also accept -t / --t spellings
        const char* val = argv[i + 1];
        try {
            switch (key[0]) {
                case 'i': in = val; break;
                case 'o': out = val; break;
                case 't': o->threshold = std::stof(val); break;
                case 'w': o->word_length = std::stoi(val); break;
                case 'd': o->drop = std::stoi(val); drop_key = true; break;
                case 'p': o->pigeon = std::stoi(val); pigeon_key = true; break;
                case 'b': o->batch = std::stoi(val); break;  // extension: tentatives per pass
                case 'g': o->device = std::stoi(val); break;  // extension: CUDA device
                case 'v': o->variant = std::stoi(val); break;  // extension: semantics
                default: return gsdr::fail(GSDR_EINVAL, "unknown option");
            }
        } catch (...) {
            return gsdr::fail(GSDR_EINVAL, "option value does not parse");
        }
    }
    if (o->variant == 1 && (drop_key || pigeon_key))
        return gsdr::fail(GSDR_EINVAL, "unknown option");  // func.cpp:27-29: usage
    if ((int64_t)in.size() + 1 > cap || (int64_t)out.size() + 1 > cap)
        return gsdr::fail(GSDR_EINVAL, "path too long");
    std::memcpy(in_path, in.c_str(), in.size() + 1);
    std::memcpy(out_path, out.c_str(), out.size() + 1);
    return gsdr_resolve_opts(o, nullptr);
}

}  // extern "C"
