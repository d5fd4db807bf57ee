// Saved acquisitions and images: the subset of HDF5 that the reference reads
// and writes (src/util/HDF5Util.h:181-287 through HDF5Util::load/save; files of
// SavedSTAAcquisition, src/user/acquisition/SavedSTAAcquisition.h:80-90, and
// Project::saveImageToHDF5, src/Project.h:106-113): one rank-1 or rank-2
// floating-point dataset per file, stored contiguous, compact or chunked, with
// the shuffle, deflate, LZF and Fletcher-32 filters. Written from the public
// HDF5 file format specification (superblock versions 0 and 1, version-1
// object headers, version-1 B-trees, local heaps, symbol table nodes).
//
// Reading: superblock -> root group (symbol table: B-tree of symbol table
// nodes, names in the local heap) -> dataset object header (dataspace,
// datatype, filter pipeline, layout) -> data (chunk B-tree for chunked
// layouts, each chunk through the filters in reverse order).
// Writing: the layout libhdf5 gives a version-0 file with one dataset:
// superblock, root group object header with its symbol table, B-tree node,
// symbol table node, local heap, dataset object header, contiguous IEEE
// little-endian 64-bit data.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/usgb.h"

namespace {

thread_local std::string g_h5Error;

struct H5Failure {
	int code;
	std::string msg;
};

#define H5_FAIL(CODE, STREAM_EXPR)          \
	do {                                    \
		std::ostringstream os_;             \
		os_ << STREAM_EXPR;                 \
		throw H5Failure{(CODE), os_.str()}; \
	} while (0)

constexpr uint64_t kUndef = ~0ULL;

// ---------------------------------------------------------------------------
// Decompressors.
// ---------------------------------------------------------------------------

// DEFLATE (RFC 1951) inside a zlib stream (RFC 1950).
class Inflater {
public:
	Inflater(const uint8_t* in, size_t n) : in_(in), n_(n) {}

	std::vector<uint8_t> run(size_t expected)
	{
		if (n_ < 2) H5_FAIL(USGB_ERR_INVALID_VALUE, "zlib stream too short");
		const unsigned cmf = in_[0], flg = in_[1];
		if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "not a zlib deflate stream");
		}
		pos_ = 2;
		out_.reserve(expected);
		bool last = false;
		while (!last) {
			last = bits(1) != 0;
			const unsigned type = bits(2);
			if (type == 0) {
				stored();
			} else if (type == 1) {
				fixed_tables();
				codes();
			} else if (type == 2) {
				dynamic_tables();
				codes();
			} else {
				H5_FAIL(USGB_ERR_INVALID_VALUE, "invalid deflate block type");
			}
		}
		return std::move(out_);
	}

private:
	struct Huffman {
		uint16_t count[16];
		std::vector<uint16_t> symbol;
	};

	unsigned bits(int need)
	{
		while (bitCount_ < need) {
			if (pos_ >= n_) H5_FAIL(USGB_ERR_INVALID_VALUE, "deflate stream truncated");
			bitBuf_ |= static_cast<uint32_t>(in_[pos_++]) << bitCount_;
			bitCount_ += 8;
		}
		const unsigned v = bitBuf_ & ((1u << need) - 1u);
		bitBuf_ >>= need;
		bitCount_ -= need;
		return v;
	}

	void stored()
	{
		bitBuf_ = 0;
		bitCount_ = 0;
		if (pos_ + 4 > n_) H5_FAIL(USGB_ERR_INVALID_VALUE, "deflate stream truncated");
		const unsigned len = in_[pos_] | (in_[pos_ + 1] << 8);
		const unsigned nlen = in_[pos_ + 2] | (in_[pos_ + 3] << 8);
		pos_ += 4;
		if ((len ^ 0xFFFFu) != nlen) H5_FAIL(USGB_ERR_INVALID_VALUE, "bad stored block length");
		if (pos_ + len > n_) H5_FAIL(USGB_ERR_INVALID_VALUE, "deflate stream truncated");
		out_.insert(out_.end(), in_ + pos_, in_ + pos_ + len);
		pos_ += len;
	}

	static void build(Huffman& h, const uint8_t* lengths, int n)
	{
		std::memset(h.count, 0, sizeof(h.count));
		for (int i = 0; i < n; ++i) h.count[lengths[i]]++;
		h.count[0] = 0;
		uint16_t offs[16];
		offs[1] = 0;
		for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
		h.symbol.assign(n, 0);
		for (int i = 0; i < n; ++i) {
			if (lengths[i]) h.symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
		}
	}

	int decode(const Huffman& h)
	{
		int code = 0, first = 0, index = 0;
		for (int len = 1; len < 16; ++len) {
			code |= static_cast<int>(bits(1));
			const int count = h.count[len];
			if (code - count < first) return h.symbol[index + (code - first)];
			index += count;
			first += count;
			first <<= 1;
			code <<= 1;
		}
		H5_FAIL(USGB_ERR_INVALID_VALUE, "invalid Huffman code");
	}

	void fixed_tables()
	{
		uint8_t l[320];
		int i = 0;
		for (; i < 144; ++i) l[i] = 8;
		for (; i < 256; ++i) l[i] = 9;
		for (; i < 280; ++i) l[i] = 7;
		for (; i < 288; ++i) l[i] = 8;
		build(lit_, l, 288);
		for (i = 0; i < 30; ++i) l[i] = 5;
		build(dist_, l, 30);
	}

	void dynamic_tables()
	{
		static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
		const int nlen = static_cast<int>(bits(5)) + 257;
		const int ndist = static_cast<int>(bits(5)) + 1;
		const int ncode = static_cast<int>(bits(4)) + 4;
		if (nlen > 286 || ndist > 30) H5_FAIL(USGB_ERR_INVALID_VALUE, "bad dynamic block counts");
		uint8_t l[320] = {0};
		for (int i = 0; i < ncode; ++i) l[order[i]] = static_cast<uint8_t>(bits(3));
		Huffman lencode;
		build(lencode, l, 19);
		int i = 0;
		uint8_t lengths[320] = {0};
		while (i < nlen + ndist) {
			int sym = decode(lencode);
			if (sym < 16) {
				lengths[i++] = static_cast<uint8_t>(sym);
			} else {
				int len = 0, rep;
				if (sym == 16) {
					if (i == 0) H5_FAIL(USGB_ERR_INVALID_VALUE, "repeat with no first length");
					len = lengths[i - 1];
					rep = 3 + static_cast<int>(bits(2));
				} else if (sym == 17) {
					rep = 3 + static_cast<int>(bits(3));
				} else {
					rep = 11 + static_cast<int>(bits(7));
				}
				if (i + rep > nlen + ndist) H5_FAIL(USGB_ERR_INVALID_VALUE, "too many code lengths");
				while (rep--) lengths[i++] = static_cast<uint8_t>(len);
			}
		}
		build(lit_, lengths, nlen);
		build(dist_, lengths + nlen, ndist);
	}

	void codes()
	{
		static const uint16_t lbase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67,
		                                   83, 99, 115, 131, 163, 195, 227, 258};
		static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5,
		                                 5, 0};
		static const uint16_t dbase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
		                                   1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
		static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
		                                 12, 12, 13, 13};
		for (;;) {
			int sym = decode(lit_);
			if (sym < 256) {
				out_.push_back(static_cast<uint8_t>(sym));
			} else if (sym == 256) {
				return;
			} else {
				sym -= 257;
				if (sym >= 29) H5_FAIL(USGB_ERR_INVALID_VALUE, "bad length symbol");
				const size_t len = lbase[sym] + bits(lext[sym]);
				const int ds = decode(dist_);
				if (ds >= 30) H5_FAIL(USGB_ERR_INVALID_VALUE, "bad distance symbol");
				const size_t dist = dbase[ds] + bits(dext[ds]);
				if (dist > out_.size()) H5_FAIL(USGB_ERR_INVALID_VALUE, "distance beyond the output");
				const size_t from = out_.size() - dist;
				for (size_t k = 0; k < len; ++k) out_.push_back(out_[from + k]);
			}
		}
	}

	const uint8_t* in_;
	size_t n_;
	size_t pos_ = 0;
	uint32_t bitBuf_ = 0;
	int bitCount_ = 0;
	Huffman lit_, dist_;
	std::vector<uint8_t> out_;
};

// LZF (the format of liblzf, used by h5py's LZF filter): a control byte c < 32
// copies c + 1 literal bytes; otherwise a back reference of length
// (c >> 5) + 2 (+ an extra byte when c >> 5 == 7) at distance
// ((c & 31) << 8) + next byte + 1.
std::vector<uint8_t> lzf_decompress(const uint8_t* in, size_t n, size_t outSize)
{
	std::vector<uint8_t> out;
	out.reserve(outSize);
	size_t i = 0;
	while (i < n) {
		const unsigned c = in[i++];
		if (c < 32) {
			const size_t len = c + 1;
			if (i + len > n) H5_FAIL(USGB_ERR_INVALID_VALUE, "LZF literal run truncated");
			out.insert(out.end(), in + i, in + i + len);
			i += len;
		} else {
			size_t len = c >> 5;
			if (len == 7) {
				if (i >= n) H5_FAIL(USGB_ERR_INVALID_VALUE, "LZF stream truncated");
				len += in[i++];
			}
			if (i >= n) H5_FAIL(USGB_ERR_INVALID_VALUE, "LZF stream truncated");
			const size_t dist = ((c & 31u) << 8) + in[i++] + 1;
			if (dist > out.size()) H5_FAIL(USGB_ERR_INVALID_VALUE, "LZF reference beyond the output");
			const size_t from = out.size() - dist;
			for (size_t k = 0; k < len + 2; ++k) out.push_back(out[from + k]);
		}
		if (out.size() > outSize) H5_FAIL(USGB_ERR_INVALID_VALUE, "LZF output larger than the chunk");
	}
	return out;
}

// ---------------------------------------------------------------------------
// Reader.
// ---------------------------------------------------------------------------
struct Dataset {
	unsigned rank = 0;
	uint64_t dims[2] = {1, 1};
	unsigned elemSize = 0;
	bool bigEndian = false;
	int layoutClass = -1;            // 0 compact, 1 contiguous, 2 chunked
	uint64_t dataAddr = kUndef, dataSize = 0;
	std::vector<uint8_t> compact;
	unsigned chunkRank = 0;          // rank + 1
	uint32_t chunkDims[3] = {0, 0, 0};
	struct Filter { unsigned id; std::vector<uint32_t> cd; };
	std::vector<Filter> filters;
};

class Reader {
public:
	explicit Reader(const std::string& path) : path_(path)
	{
		std::ifstream f(path, std::ios::binary);
		if (!f) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "Could not open the file " << path << '.');
		f.seekg(0, std::ios::end);
		const std::streamoff size = f.tellg();
		if (size <= 0) H5_FAIL(USGB_ERR_INVALID_VALUE, "Empty file " << path << '.');
		f.seekg(0);
		buf_.resize(static_cast<size_t>(size));
		f.read(reinterpret_cast<char*>(buf_.data()), size);
		if (!f) H5_FAIL(USGB_ERR_INVALID_VALUE, "Could not read the file " << path << '.');
		superblock();
	}

	Dataset open(const std::string& name)
	{
		const uint64_t oh = find_in_root(name);
		Dataset d;
		read_header(oh, d);
		if (d.rank == 0 || d.rank > 2) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "The rank in the file " << path_ << " is not 1 or 2.");
		}
		if (d.elemSize != 4 && d.elemSize != 8) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "The data type in the file " << path_ << " is not 32- or 64-bit floating point.");
		}
		if (d.layoutClass < 0) H5_FAIL(USGB_ERR_INVALID_VALUE, "No data layout in the file " << path_ << '.');
		return d;
	}

	// Row-major doubles.
	std::vector<double> read(const Dataset& d)
	{
		const uint64_t n = d.dims[0] * (d.rank == 2 ? d.dims[1] : 1);
		std::vector<uint8_t> raw(n * d.elemSize, 0);
		if (d.layoutClass == 0) {
			if (d.compact.size() < raw.size()) H5_FAIL(USGB_ERR_INVALID_VALUE, "Compact data too short in " << path_ << '.');
			std::memcpy(raw.data(), d.compact.data(), raw.size());
		} else if (d.layoutClass == 1) {
			if (d.dataAddr != kUndef) {
				need(d.dataAddr, raw.size());
				std::memcpy(raw.data(), &buf_[d.dataAddr], raw.size());
			}
		} else {
			read_chunks(d, raw);
		}
		std::vector<double> out(n);
		for (uint64_t i = 0; i < n; ++i) {
			uint8_t b[8];
			std::memcpy(b, &raw[i * d.elemSize], d.elemSize);
			if (d.bigEndian) std::reverse(b, b + d.elemSize);
			if (d.elemSize == 8) {
				double v;
				std::memcpy(&v, b, 8);
				out[i] = v;
			} else {
				float v;
				std::memcpy(&v, b, 4);
				out[i] = v;
			}
		}
		return out;
	}

private:
	void need(uint64_t off, uint64_t len) const
	{
		if (off > buf_.size() || len > buf_.size() - off) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "Truncated or corrupt file " << path_ << '.');
		}
	}
	uint64_t u(uint64_t off, unsigned len) const
	{
		need(off, len);
		uint64_t v = 0;
		for (unsigned i = 0; i < len; ++i) v |= static_cast<uint64_t>(buf_[off + i]) << (8 * i);
		if (len == 8 && v == kUndef) return kUndef;
		return v;
	}
	uint64_t addr(uint64_t off) const
	{
		const uint64_t a = u(off, so_);
		if (so_ < 8 && a == (1ULL << (8 * so_)) - 1ULL) return kUndef;
		return a == kUndef ? kUndef : a + base_;
	}

	void superblock()
	{
		static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
		uint64_t at = kUndef;
		for (uint64_t o = 0; o + 8 <= buf_.size(); o = (o == 0 ? 512 : o * 2)) {
			if (std::memcmp(&buf_[o], sig, 8) == 0) {
				at = o;
				break;
			}
		}
		if (at == kUndef) H5_FAIL(USGB_ERR_INVALID_VALUE, "The file " << path_ << " is not an HDF5 file.");
		need(at, 24);
		const unsigned version = buf_[at + 8];
		if (version > 1) {
			H5_FAIL(USGB_ERR_UNSUPPORTED, "HDF5 superblock version " << version << " in " << path_
					<< " (versions 0 and 1 are read).");
		}
		so_ = buf_[at + 13];
		sl_ = buf_[at + 14];
		if (so_ != 8 && so_ != 4) H5_FAIL(USGB_ERR_UNSUPPORTED, "HDF5 offset size " << so_ << " in " << path_ << '.');
		if (sl_ != 8 && sl_ != 4) H5_FAIL(USGB_ERR_UNSUPPORTED, "HDF5 length size " << sl_ << " in " << path_ << '.');
		groupLeafK_ = static_cast<unsigned>(u(at + 16, 2));
		uint64_t p = at + 24;
		if (version == 1) p += 4;   // indexed storage internal node K, reserved
		base_ = u(p, so_);
		p += 4 * so_;               // base, free space, end of file, driver info
		// Root group symbol table entry: link name offset, object header address, cache type, scratch.
		rootHeader_ = addr(p + so_);
		const uint64_t cache = u(p + 2 * so_, 4);
		if (cache == 1) {
			rootBtree_ = addr(p + 2 * so_ + 8);
			rootHeap_ = addr(p + 3 * so_ + 8);
		}
	}

	// Iterates the messages of a version-1 object header (and its continuations).
	template<typename F>
	void messages(uint64_t oh, F&& f)
	{
		need(oh, 16);
		if (buf_[oh] != 1) {
			H5_FAIL(USGB_ERR_UNSUPPORTED, "HDF5 object header version " << unsigned(buf_[oh]) << " in " << path_ << '.');
		}
		const unsigned total = static_cast<unsigned>(u(oh + 2, 2));
		std::vector<std::pair<uint64_t, uint64_t>> blocks = {{oh + 16, u(oh + 8, 4)}};
		unsigned seen = 0;
		for (size_t bi = 0; bi < blocks.size() && bi < 64; ++bi) {
			uint64_t p = blocks[bi].first;
			const uint64_t end = p + blocks[bi].second;
			need(blocks[bi].first, blocks[bi].second);
			while (p + 8 <= end && seen < total) {
				const unsigned type = static_cast<unsigned>(u(p, 2));
				const unsigned size = static_cast<unsigned>(u(p + 2, 2));
				need(p + 8, size);
				if (type == 0x10) {
					blocks.push_back({addr(p + 8), u(p + 8 + so_, sl_)});
				} else {
					f(type, p + 8, size);
				}
				++seen;
				p += 8 + size;
			}
		}
	}

	uint64_t find_in_root(const std::string& name)
	{
		if (rootBtree_ == kUndef || rootHeap_ == kUndef) {
			messages(rootHeader_, [&](unsigned type, uint64_t p, unsigned) {
				if (type == 0x11) {
					rootBtree_ = addr(p);
					rootHeap_ = addr(p + so_);
				}
			});
		}
		if (rootBtree_ == kUndef || rootHeap_ == kUndef) {
			H5_FAIL(USGB_ERR_UNSUPPORTED, "The root group of " << path_ << " has no symbol table.");
		}
		need(rootHeap_, 8 + 2 * sl_ + so_);
		if (std::memcmp(&buf_[rootHeap_], "HEAP", 4) != 0) H5_FAIL(USGB_ERR_INVALID_VALUE, "Bad local heap in " << path_ << '.');
		const uint64_t heapSize = u(rootHeap_ + 8, sl_);
		const uint64_t heapData = addr(rootHeap_ + 8 + 2 * sl_);
		need(heapData, heapSize);
		uint64_t found = kUndef;
		walk_group(rootBtree_, heapData, heapSize, name, found, 0);
		if (found == kUndef) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "No dataset \"" << name << "\" in the file " << path_ << '.');
		return found;
	}

	void walk_group(uint64_t node, uint64_t heapData, uint64_t heapSize, const std::string& name, uint64_t& found, int depth)
	{
		if (depth > 32) H5_FAIL(USGB_ERR_INVALID_VALUE, "Group B-tree too deep in " << path_ << '.');
		need(node, 8 + 2 * so_);
		if (std::memcmp(&buf_[node], "TREE", 4) != 0 || buf_[node + 4] != 0) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "Bad group B-tree node in " << path_ << '.');
		}
		const unsigned level = buf_[node + 5];
		const unsigned used = static_cast<unsigned>(u(node + 6, 2));
		uint64_t p = node + 8 + 2 * so_ + sl_;   // first child (after key 0)
		for (unsigned i = 0; i < used && found == kUndef; ++i) {
			const uint64_t child = addr(p);
			if (level > 0) {
				walk_group(child, heapData, heapSize, name, found, depth + 1);
			} else {
				need(child, 8);
				if (std::memcmp(&buf_[child], "SNOD", 4) != 0) H5_FAIL(USGB_ERR_INVALID_VALUE, "Bad symbol table node in " << path_ << '.');
				const unsigned nsym = static_cast<unsigned>(u(child + 6, 2));
				const unsigned entry = 2 * so_ + 24;
				for (unsigned k = 0; k < nsym; ++k) {
					const uint64_t e = child + 8 + static_cast<uint64_t>(k) * entry;
					const uint64_t nameOff = u(e, so_);
					if (nameOff >= heapSize) H5_FAIL(USGB_ERR_INVALID_VALUE, "Bad link name in " << path_ << '.');
					const char* s = reinterpret_cast<const char*>(&buf_[heapData + nameOff]);
					const size_t maxLen = heapSize - nameOff;
					if (strnlen(s, maxLen) == name.size() && std::memcmp(s, name.data(), name.size()) == 0) {
						found = addr(e + so_);
						break;
					}
				}
			}
			p += so_ + sl_;
		}
	}

	void read_header(uint64_t oh, Dataset& d)
	{
		messages(oh, [&](unsigned type, uint64_t p, unsigned size) {
			switch (type) {
			case 0x01: {  // dataspace
				const unsigned version = buf_[p];
				d.rank = buf_[p + 1];
				if (d.rank > 2) return;
				const uint64_t dimsAt = p + (version == 1 ? 8 : 4);
				for (unsigned i = 0; i < d.rank; ++i) d.dims[i] = u(dimsAt + i * sl_, sl_);
				break;
			}
			case 0x03: {  // datatype
				const unsigned cls = buf_[p] & 15u;
				if (cls != 1) H5_FAIL(USGB_ERR_INVALID_VALUE, "The data type class in the file " << path_ << " is not floating point.");
				d.bigEndian = (buf_[p + 1] & 1u) != 0;
				d.elemSize = static_cast<unsigned>(u(p + 4, 4));
				break;
			}
			case 0x08: {  // data layout
				const unsigned version = buf_[p];
				if (version == 3) {
					d.layoutClass = buf_[p + 1];
					if (d.layoutClass == 0) {
						const unsigned n = static_cast<unsigned>(u(p + 2, 2));
						need(p + 4, n);
						d.compact.assign(&buf_[p + 4], &buf_[p + 4] + n);
					} else if (d.layoutClass == 1) {
						d.dataAddr = addr(p + 2);
						d.dataSize = u(p + 2 + so_, sl_);
					} else if (d.layoutClass == 2) {
						d.chunkRank = buf_[p + 2];
						d.dataAddr = addr(p + 3);
						if (d.chunkRank < 2 || d.chunkRank > 3) H5_FAIL(USGB_ERR_UNSUPPORTED, "Chunk rank in " << path_ << '.');
						for (unsigned i = 0; i < d.chunkRank; ++i) d.chunkDims[i] = static_cast<uint32_t>(u(p + 3 + so_ + 4 * i, 4));
					} else {
						H5_FAIL(USGB_ERR_UNSUPPORTED, "Layout class " << d.layoutClass << " in " << path_ << '.');
					}
				} else if (version == 1 || version == 2) {
					const unsigned dimsN = buf_[p + 1];
					d.layoutClass = buf_[p + 2];
					uint64_t q = p + 8;
					if (d.layoutClass != 0) {
						d.dataAddr = addr(q);
						q += so_;
					}
					if (d.layoutClass == 2) {
						d.chunkRank = dimsN;
						if (dimsN < 2 || dimsN > 3) H5_FAIL(USGB_ERR_UNSUPPORTED, "Chunk rank in " << path_ << '.');
						for (unsigned i = 0; i < dimsN; ++i) d.chunkDims[i] = static_cast<uint32_t>(u(q + 4 * i, 4));
					} else if (d.layoutClass == 0) {
						const uint64_t c = q + 4 * dimsN;
						const unsigned n = static_cast<unsigned>(u(c, 4));
						need(c + 4, n);
						d.compact.assign(&buf_[c + 4], &buf_[c + 4] + n);
					}
				} else {
					H5_FAIL(USGB_ERR_UNSUPPORTED, "Layout message version " << version << " in " << path_ << '.');
				}
				break;
			}
			case 0x0B: {  // filter pipeline
				const unsigned version = buf_[p];
				const unsigned nf = buf_[p + 1];
				uint64_t q = p + (version == 1 ? 8 : 2);
				for (unsigned i = 0; i < nf; ++i) {
					Dataset::Filter f;
					f.id = static_cast<unsigned>(u(q, 2));
					unsigned nameLen = 0;
					if (version == 1 || f.id >= 256) {
						nameLen = static_cast<unsigned>(u(q + 2, 2));
						q += 2;
					}
					const unsigned ncd = static_cast<unsigned>(u(q + 4, 2));
					q += 6;
					if (version == 1) nameLen = (nameLen + 7u) & ~7u;
					q += nameLen;
					for (unsigned k = 0; k < ncd; ++k) f.cd.push_back(static_cast<uint32_t>(u(q + 4 * k, 4)));
					q += 4 * ncd;
					if (version == 1 && (ncd & 1u)) q += 4;
					d.filters.push_back(f);
				}
				(void)size;
				break;
			}
			default:
				break;
			}
		});
	}

	void collect_chunks(uint64_t node, unsigned ndims, std::vector<std::pair<std::vector<uint64_t>, std::vector<uint64_t>>>& out,
			int depth)
	{
		// out: (offsets, {size, filterMask, address})
		if (depth > 32) H5_FAIL(USGB_ERR_INVALID_VALUE, "Chunk B-tree too deep in " << path_ << '.');
		need(node, 8 + 2 * so_);
		if (std::memcmp(&buf_[node], "TREE", 4) != 0 || buf_[node + 4] != 1) {
			H5_FAIL(USGB_ERR_INVALID_VALUE, "Bad chunk B-tree node in " << path_ << '.');
		}
		const unsigned level = buf_[node + 5];
		const unsigned used = static_cast<unsigned>(u(node + 6, 2));
		const unsigned keySize = 8 + 8 * ndims;
		uint64_t p = node + 8 + 2 * so_;
		for (unsigned i = 0; i < used; ++i) {
			const uint64_t size = u(p, 4);
			const uint64_t mask = u(p + 4, 4);
			std::vector<uint64_t> offs(ndims);
			for (unsigned k = 0; k < ndims; ++k) offs[k] = u(p + 8 + 8 * k, 8);
			const uint64_t child = addr(p + keySize);
			if (level > 0) {
				collect_chunks(child, ndims, out, depth + 1);
			} else {
				out.push_back({offs, {size, mask, child}});
			}
			p += keySize + so_;
		}
	}

	void read_chunks(const Dataset& d, std::vector<uint8_t>& raw)
	{
		if (d.dataAddr == kUndef) return;  // never written: fill value 0
		std::vector<std::pair<std::vector<uint64_t>, std::vector<uint64_t>>> chunks;
		collect_chunks(d.dataAddr, d.chunkRank, chunks, 0);
		const unsigned rank = d.rank;
		const uint64_t c0 = d.chunkDims[0], c1 = rank == 2 ? d.chunkDims[1] : 1;
		const uint64_t elem = d.chunkDims[rank];
		if (elem != d.elemSize) H5_FAIL(USGB_ERR_INVALID_VALUE, "Chunk element size mismatch in " << path_ << '.');
		const uint64_t chunkBytes = c0 * c1 * elem;
		const uint64_t n0 = d.dims[0], n1 = rank == 2 ? d.dims[1] : 1;
		for (const auto& ch : chunks) {
			const uint64_t size = ch.second[0], mask = ch.second[1], at = ch.second[2];
			need(at, size);
			std::vector<uint8_t> data(&buf_[at], &buf_[at] + size);
			for (size_t fi = d.filters.size(); fi-- > 0;) {
				if (mask & (1ULL << fi)) continue;
				const Dataset::Filter& f = d.filters[fi];
				if (f.id == 1) {
					data = Inflater(data.data(), data.size()).run(chunkBytes);
				} else if (f.id == 2) {
					const size_t es = f.cd.empty() ? elem : f.cd[0];
					if (es > 1 && data.size() % es == 0) {
						std::vector<uint8_t> t(data.size());
						const size_t n = data.size() / es;
						for (size_t b = 0; b < es; ++b) {
							for (size_t i = 0; i < n; ++i) t[i * es + b] = data[b * n + i];
						}
						data.swap(t);
					}
				} else if (f.id == 3) {
					if (data.size() < 4) H5_FAIL(USGB_ERR_INVALID_VALUE, "Fletcher-32 chunk too short in " << path_ << '.');
					data.resize(data.size() - 4);
				} else if (f.id == 32000) {
					data = lzf_decompress(data.data(), data.size(), chunkBytes);
				} else {
					H5_FAIL(USGB_ERR_UNSUPPORTED, "HDF5 filter " << f.id << " in " << path_ << " is not supported.");
				}
			}
			if (data.size() < chunkBytes) H5_FAIL(USGB_ERR_INVALID_VALUE, "Short chunk in " << path_ << '.');
			const uint64_t o0 = ch.first[0], o1 = rank == 2 ? ch.first[1] : 0;
			for (uint64_t i = 0; i < c0 && o0 + i < n0; ++i) {
				const uint64_t cols = std::min<uint64_t>(c1, n1 > o1 ? n1 - o1 : 0);
				if (cols == 0) continue;
				std::memcpy(&raw[((o0 + i) * n1 + o1) * elem], &data[(i * c1) * elem], cols * elem);
			}
		}
	}

	std::string path_;
	std::vector<uint8_t> buf_;
	unsigned so_ = 8, sl_ = 8, groupLeafK_ = 4;
	uint64_t base_ = 0, rootHeader_ = kUndef, rootBtree_ = kUndef, rootHeap_ = kUndef;
};

// ---------------------------------------------------------------------------
// Writer: one contiguous IEEE 64-bit little-endian dataset in a version-0 file.
// ---------------------------------------------------------------------------
class Writer {
public:
	void put(uint64_t v, unsigned n) { for (unsigned i = 0; i < n; ++i) b_.push_back(static_cast<uint8_t>(v >> (8 * i))); }
	void bytes(const void* p, size_t n) { const auto* c = static_cast<const uint8_t*>(p); b_.insert(b_.end(), c, c + n); }
	void zeros(size_t n) { b_.insert(b_.end(), n, 0); }
	void align8() { while (b_.size() % 8) b_.push_back(0); }
	void patch(size_t at, uint64_t v, unsigned n) { for (unsigned i = 0; i < n; ++i) b_[at + i] = static_cast<uint8_t>(v >> (8 * i)); }
	size_t size() const { return b_.size(); }
	const std::vector<uint8_t>& data() const { return b_; }
private:
	std::vector<uint8_t> b_;
};

// Object header message (version-1 header): type, size padded to 8, flags.
void message(Writer& w, unsigned type, const Writer& body, unsigned flags = 0)
{
	const size_t n = (body.size() + 7u) & ~size_t(7);
	w.put(type, 2);
	w.put(n, 2);
	w.put(flags, 1);
	w.zeros(3);
	w.bytes(body.data().data(), body.size());
	w.zeros(n - body.size());
}

std::vector<uint8_t> write_file(const std::string& name, const double* data, uint64_t n1, uint64_t n2)
{
	constexpr unsigned K_LEAF = 4, K_INTERNAL = 16;
	Writer w;
	// Superblock (version 0), 96 bytes; addresses patched below.
	static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
	w.bytes(sig, 8);
	w.put(0, 1); w.put(0, 1); w.put(0, 1); w.put(0, 1);   // superblock, free space, root entry, reserved
	w.put(0, 1); w.put(8, 1); w.put(8, 1); w.put(0, 1);   // shared header version, offset size, length size
	w.put(K_LEAF, 2); w.put(K_INTERNAL, 2);
	w.put(0, 4);                                           // consistency flags
	w.put(0, 8);                                           // base address
	w.put(kUndef, 8);                                      // free-space info
	const size_t eofAt = w.size();
	w.put(0, 8);                                           // end of file
	w.put(kUndef, 8);                                      // driver information
	// Root group symbol table entry.
	w.put(0, 8);                                           // link name offset ("")
	const size_t rootOhAt = w.size();
	w.put(0, 8);
	w.put(1, 4);                                           // cache type 1: B-tree and heap addresses follow
	w.put(0, 4);
	const size_t rootScratch = w.size();
	w.put(0, 8);
	w.put(0, 8);

	// Root group object header: symbol table message.
	const size_t rootOh = w.size();
	Writer stab;
	stab.put(0, 8);
	stab.put(0, 8);
	w.put(1, 1); w.put(0, 1); w.put(1, 2);                 // version, reserved, 1 message
	w.put(1, 4);                                           // reference count
	w.put(8 + 16, 4);                                      // header data size
	w.put(0, 4);                                           // alignment
	const size_t stabAt = w.size() + 8;
	message(w, 0x11, stab);
	w.patch(rootOhAt, rootOh, 8);

	// Group B-tree (type 0, one leaf entry), sized for 2 * K_INTERNAL entries.
	const size_t btree = w.size();
	w.bytes("TREE", 4);
	w.put(0, 1); w.put(0, 1); w.put(1, 2);
	w.put(kUndef, 8); w.put(kUndef, 8);
	w.put(0, 8);                                           // key 0: ""
	const size_t childAt = w.size();
	w.put(0, 8);                                           // child 0: symbol table node
	const size_t key1At = w.size();
	w.put(0, 8);                                           // key 1: the dataset name
	w.zeros((2 * K_INTERNAL - 1) * 16);

	// Local heap: "" at 0, then the name; 8-byte padded.
	std::vector<uint8_t> heapData(8, 0);
	const size_t nameOff = heapData.size();
	heapData.insert(heapData.end(), name.begin(), name.end());
	heapData.push_back(0);
	while (heapData.size() % 8) heapData.push_back(0);
	const size_t heap = w.size();
	w.bytes("HEAP", 4);
	w.put(0, 1); w.zeros(3);
	w.put(heapData.size(), 8);
	w.put(kUndef, 8);                                      // no free block
	const size_t heapDataAddrAt = w.size();
	w.put(0, 8);
	const size_t heapDataAddr = w.size();
	w.bytes(heapData.data(), heapData.size());
	w.patch(heapDataAddrAt, heapDataAddr, 8);
	w.patch(key1At, nameOff, 8);

	// Symbol table node with the dataset entry, sized for 2 * K_LEAF entries.
	const size_t snod = w.size();
	w.bytes("SNOD", 4);
	w.put(1, 1); w.put(0, 1); w.put(1, 2);
	w.put(nameOff, 8);
	const size_t dsOhAt = w.size();
	w.put(0, 8);
	w.put(0, 4); w.put(0, 4);
	w.zeros(16);
	w.zeros((2 * K_LEAF - 1) * 40);
	w.patch(childAt, snod, 8);

	// Dataset object header: dataspace, datatype, fill value, layout.
	w.align8();
	const size_t dsOh = w.size();
	Writer space, type, fill, layout;
	space.put(1, 1); space.put(2, 1); space.put(0, 1); space.put(0, 1); space.put(0, 4);
	space.put(n1, 8); space.put(n2, 8);
	type.put(0x11, 1);                                     // version 1, class 1 (floating point)
	type.put(0x20, 1); type.put(63, 1); type.put(0, 1);    // little-endian, implied mantissa MSB; sign bit 63
	type.put(8, 4);
	type.put(0, 2); type.put(64, 2);                       // bit offset, precision
	type.put(52, 1); type.put(11, 1); type.put(0, 1); type.put(52, 1);
	type.put(1023, 4);
	fill.put(2, 1); fill.put(1, 1); fill.put(0, 1); fill.put(0, 1);   // version 2, early allocation, write on alloc, undefined
	layout.put(3, 1); layout.put(1, 1);                    // version 3, contiguous
	layout.put(0, 8);                                      // data address (patched)
	layout.put(n1 * n2 * 8, 8);
	const size_t msgBytes = (8 + ((space.size() + 7) & ~size_t(7))) + (8 + ((type.size() + 7) & ~size_t(7))) +
			(8 + ((fill.size() + 7) & ~size_t(7))) + (8 + ((layout.size() + 7) & ~size_t(7)));
	w.put(1, 1); w.put(0, 1); w.put(4, 2);
	w.put(1, 4);
	w.put(msgBytes, 4);
	w.put(0, 4);
	message(w, 0x01, space);
	message(w, 0x03, type, 1);                             // constant
	message(w, 0x05, fill, 1);
	const size_t layoutBody = w.size() + 8;
	message(w, 0x08, layout);
	w.patch(dsOhAt, dsOh, 8);

	// Data.
	w.align8();
	const size_t dataAt = w.size();
	for (uint64_t i = 0; i < n1 * n2; ++i) {
		uint64_t bits;
		std::memcpy(&bits, &data[i], 8);
		w.put(bits, 8);
	}
	w.patch(layoutBody + 2, dataAt, 8);

	w.patch(stabAt, btree, 8);
	w.patch(stabAt + 8, heap, 8);
	w.patch(rootScratch, btree, 8);
	w.patch(rootScratch + 8, heap, 8);
	w.patch(eofAt, w.size(), 8);
	return w.data();
}

template<typename F>
int h5_guarded(F&& f)
{
	try {
		f();
		return USGB_OK;
	} catch (const H5Failure& e) {
		g_h5Error = e.msg;
		return e.code;
	} catch (const std::bad_alloc&) {
		g_h5Error = "host allocation failed";
		return USGB_ERR_OUT_OF_MEMORY;
	} catch (const std::exception& e) {
		g_h5Error = e.what();
		return USGB_ERR_INVALID_STATE;
	}
}

}  // namespace

extern "C" {

const char* usgb_h5_last_error(void) { return g_h5Error.c_str(); }

int usgb_h5_dataset_info(const char* path, const char* dataset, uint32_t* rank, uint64_t* n1, uint64_t* n2)
{
	return h5_guarded([&] {
		if (!path || !dataset) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "null path or dataset name");
		Reader r(path);
		const Dataset d = r.open(dataset);
		if (rank) *rank = d.rank;
		if (n1) *n1 = d.rank == 2 ? d.dims[0] : 1;
		if (n2) *n2 = d.rank == 2 ? d.dims[1] : d.dims[0];
	});
}

int usgb_h5_read_f64(const char* path, const char* dataset, double* out, size_t capacity, uint64_t* n1, uint64_t* n2)
{
	return h5_guarded([&] {
		if (!path || !dataset) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "null path or dataset name");
		Reader r(path);
		const Dataset d = r.open(dataset);
		const uint64_t a = d.rank == 2 ? d.dims[0] : 1, b = d.rank == 2 ? d.dims[1] : d.dims[0];
		if (n1) *n1 = a;
		if (n2) *n2 = b;
		if (a * b > capacity) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "The dataset has " << a * b << " values, the buffer holds " << capacity << '.');
		if (!out) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "null output");
		const std::vector<double> v = r.read(d);
		std::memcpy(out, v.data(), v.size() * sizeof(double));
	});
}

int usgb_h5_write_f64(const char* path, const char* dataset, const double* data, uint64_t n1, uint64_t n2)
{
	return h5_guarded([&] {
		if (!path || !dataset || !data) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "null argument");
		if (n1 == 0) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "The container's first dimension (" << n1 << ") is equal to 0.");
		if (n2 == 0) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "The container's second dimension (" << n2 << ") is equal to 0.");
		const std::string name(dataset);
		if (name.empty() || name.find('/') != std::string::npos) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid dataset name.");
		const std::vector<uint8_t> file = write_file(name, data, n1, n2);
		std::ofstream f(path, std::ios::binary | std::ios::trunc);
		if (!f) H5_FAIL(USGB_ERR_INVALID_PARAMETER, "Could not create the file " << path << '.');
		f.write(reinterpret_cast<const char*>(file.data()), static_cast<std::streamsize>(file.size()));
		if (!f) H5_FAIL(USGB_ERR_INVALID_VALUE, "Could not write the file " << path << '.');
	});
}

}  // extern "C"
