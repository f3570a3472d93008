// ampfile.cpp -- raw amplitude files: the decay amplitudes of one event file
// for a set of waves plus the event file's binning variables.
//
// The reference keeps one ROOT tree of amplitudeTreeLeaf objects per wave
// (storageFormats/amplitudeTreeLeaf.h:51-118, read by
// pwaLikelihood::addAmplitude, partialWaveFit/pwaLikelihood.cc:1110-1288) and
// reads the binning variables of on-the-fly binning from the event file's
// metadata tree (pwaLikelihood.cc:1391-1440).  Here both live in one flat
// little-endian file laid out for sequential reads straight into device
// memory:
//
//   offset  size  field
//        0     8  magic "RPWAAMP" + NUL
//        8     4  format version (1)
//       12     4  number of waves W
//       16     4  number of binning variables V
//       20     4  zero
//       24     8  number of events N
//       32     8  offset of the data block (multiple of 4096)
//       40        W wave names, then V variable names: u16 length + bytes
//   data block:   W rows of N complex64 (re, im float32), one row per wave;
//                 then V rows of N float64, one row per variable.
//
// The file is N * (8 W + 8 V) bytes plus the header; a reader checks that
// the file is exactly that long.

#include "pwa_gb300.h"
#include "pwa_internal.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstring>
#include <set>

namespace pwa {

namespace {

constexpr char kMagic[8] = {'R', 'P', 'W', 'A', 'A', 'M', 'P', '\0'};
constexpr uint32_t kVersion = 1;
constexpr uint64_t kAlign = 4096;

template <typename T>
void put(std::vector<unsigned char>& b, T v)
{
	unsigned char raw[sizeof(T)];
	std::memcpy(raw, &v, sizeof(T));
	b.insert(b.end(), raw, raw + sizeof(T));
}

template <typename T>
bool get(const std::vector<unsigned char>& b, size_t& pos, T& v)
{
	if (pos + sizeof(T) > b.size())
		return false;
	std::memcpy(&v, b.data() + pos, sizeof(T));
	pos += sizeof(T);
	return true;
}

int writeAll(int fd, const void* p, size_t bytes, const char* path)
{
	const unsigned char* c = static_cast<const unsigned char*>(p);
	while (bytes > 0) {
		const ssize_t w = ::write(fd, c, bytes);
		if (w < 0) {
			if (errno == EINTR)
				continue;
			return setError(kErrIo, std::string("write failed for '") + path + "': " + std::strerror(errno));
		}
		c += w;
		bytes -= (size_t)w;
	}
	return kOk;
}

int preadAll(int fd, void* p, size_t bytes, uint64_t offset, const std::string& path)
{
	unsigned char* c = static_cast<unsigned char*>(p);
	while (bytes > 0) {
		const ssize_t r = ::pread(fd, c, bytes, (off_t)offset);
		if (r < 0) {
			if (errno == EINTR)
				continue;
			return setError(kErrIo, "read failed for '" + path + "': " + std::strerror(errno));
		}
		if (r == 0)
			return setError(kErrIo, "unexpected end of file in '" + path + "'");
		c += r;
		bytes -= (size_t)r;
		offset += (uint64_t)r;
	}
	return kOk;
}

}  // namespace

int ampFileOpen(const char* path, AmpFile& f)
{
	f = AmpFile();
	f.path = path;
	f.fd = ::open(path, O_RDONLY);
	if (f.fd < 0)
		return setError(kErrIo, std::string("cannot open amplitude file '") + path + "': " + std::strerror(errno));
	struct stat st;
	if (::fstat(f.fd, &st) != 0)
		return setError(kErrIo, std::string("cannot stat '") + path + "'");
	std::vector<unsigned char> head(40);
	if ((uint64_t)st.st_size < head.size())
		return setError(kErrIo, std::string("'") + path + "' is not an amplitude file (too short)");
	int st0 = preadAll(f.fd, head.data(), head.size(), 0, f.path);
	if (st0 != kOk)
		return st0;
	if (std::memcmp(head.data(), kMagic, 8) != 0)
		return setError(kErrIo, std::string("'") + path + "' is not an amplitude file (bad magic)");
	size_t pos = 8;
	uint32_t version = 0, zero = 0;
	get(head, pos, version);
	get(head, pos, f.nWaves);
	get(head, pos, f.nVars);
	get(head, pos, zero);
	get(head, pos, f.nEvents);
	get(head, pos, f.dataOffset);
	if (version != kVersion)
		return setError(kErrIo, std::string("'") + path + "': unsupported format version " + std::to_string(version));
	if (f.dataOffset < 40 || f.dataOffset % kAlign != 0 || f.dataOffset > (uint64_t)st.st_size)
		return setError(kErrIo, std::string("'") + path + "': bad data offset");
	std::vector<unsigned char> names(f.dataOffset - 40);
	st0 = preadAll(f.fd, names.data(), names.size(), 40, f.path);
	if (st0 != kOk)
		return st0;
	pos = 0;
	for (uint32_t i = 0; i < f.nWaves + f.nVars; ++i) {
		uint16_t len = 0;
		if (!get(names, pos, len) || pos + len > names.size())
			return setError(kErrIo, std::string("'") + path + "': truncated name table");
		std::string s(reinterpret_cast<const char*>(names.data() + pos), len);
		pos += len;
		(i < f.nWaves ? f.waves : f.vars).push_back(s);
	}
	const uint64_t expect = f.dataOffset + f.nEvents * 8ull * ((uint64_t)f.nWaves + f.nVars);
	if ((uint64_t)st.st_size != expect)
		return setError(kErrIo, std::string("'") + path + "': file size " + std::to_string((uint64_t)st.st_size) +
		                            " differs from the header's " + std::to_string(expect));
	return kOk;
}

AmpFile::~AmpFile()
{
	if (fd >= 0)
		::close(fd);
}

AmpFile& AmpFile::operator=(AmpFile&& o) noexcept
{
	if (this != &o) {
		if (fd >= 0)
			::close(fd);
		fd = o.fd;
		o.fd = -1;
		path = std::move(o.path);
		nWaves = o.nWaves;
		nVars = o.nVars;
		nEvents = o.nEvents;
		dataOffset = o.dataOffset;
		waves = std::move(o.waves);
		vars = std::move(o.vars);
	}
	return *this;
}

// file bytes [offset, offset + bytes) -> device memory, through two pinned
// staging buffers so that the read of one chunk overlaps the copy of the last
int ampFileToDevice(const AmpFile& f, uint64_t offset, uint64_t bytes, void* dst, cudaStream_t s)
{
	constexpr size_t kStage = size_t(16) << 20;
	void* stage[2] = {nullptr, nullptr};
	cudaEvent_t done[2] = {nullptr, nullptr};
	int st = kOk;
	for (int k = 0; k < 2 && st == kOk; ++k) {
		st = cudaCheck(cudaHostAlloc(&stage[k], kStage, cudaHostAllocDefault), "pinned staging");
		if (st == kOk)
			st = cudaCheck(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming), "event");
	}
	bool used[2] = {false, false};
	for (uint64_t b = 0, k = 0; st == kOk && b < bytes; b += kStage, k ^= 1) {
		const size_t m = (size_t)std::min<uint64_t>(kStage, bytes - b);
		if (used[k])
			st = cudaCheck(cudaEventSynchronize(done[k]), "staging reuse");
		if (st == kOk)
			st = preadAll(f.fd, stage[k], m, offset + b, f.path);
		if (st == kOk)
			st = cudaCheck(cudaMemcpyAsync(static_cast<unsigned char*>(dst) + b, stage[k], m, cudaMemcpyHostToDevice, s),
			               "amplitude file upload");
		if (st == kOk)
			st = cudaCheck(cudaEventRecord(done[k], s), "event record");
		used[k] = true;
	}
	const int st2 = cudaCheck(cudaStreamSynchronize(s), "amplitude file upload");
	for (int k = 0; k < 2; ++k) {
		if (done[k])
			cudaEventDestroy(done[k]);
		if (stage[k])
			cudaFreeHost(stage[k]);
	}
	return st != kOk ? st : st2;
}

}  // namespace pwa

using namespace pwa;

namespace pwa {

// header of an amplitude file up to its data block (padded to the 4096-byte
// boundary); names[0 .. nWaves) are the waves, the rest the binning variables
int ampFileHeader(uint32_t nWaves, uint32_t nVars, const char* const* names, uint64_t nEvents,
                  std::vector<unsigned char>& h)
{
	h.assign(kMagic, kMagic + 8);
	put<uint32_t>(h, kVersion);
	put<uint32_t>(h, nWaves);
	put<uint32_t>(h, nVars);
	put<uint32_t>(h, 0);
	put<uint64_t>(h, nEvents);
	put<uint64_t>(h, 0);  // data offset, filled below
	std::set<std::string> waveSet, varSet;
	for (uint32_t i = 0; i < nWaves + nVars; ++i) {
		const char* name = names[i];
		if (!name)
			return setError(kErrArg, "amplitude file: null name");
		const size_t len = std::strlen(name);
		if (len == 0 || len > 65535)
			return setError(kErrArg, "amplitude file: names must have 1..65535 bytes");
		// readers look waves and binning variables up by name
		if (!(i < nWaves ? waveSet : varSet).insert(name).second)
			return setError(kErrArg, std::string("amplitude file: duplicate ") + (i < nWaves ? "wave" : "variable") +
			                             " name '" + name + "'");
		put<uint16_t>(h, (uint16_t)len);
		h.insert(h.end(), name, name + len);
	}
	const uint64_t dataOffset = (h.size() + kAlign - 1) / kAlign * kAlign;
	std::memcpy(h.data() + 32, &dataOffset, 8);
	h.resize(dataOffset, 0);
	return kOk;
}

// bytes to file offset (pwrite, restarted on EINTR and short writes)
int ampFilePwrite(int fd, const void* p, size_t bytes, uint64_t offset, const char* path)
{
	const unsigned char* c = static_cast<const unsigned char*>(p);
	while (bytes > 0) {
		const ssize_t w = ::pwrite(fd, c, bytes, (off_t)offset);
		if (w < 0) {
			if (errno == EINTR)
				continue;
			return setError(kErrIo, std::string("write failed for '") + path + "': " + std::strerror(errno));
		}
		c += w;
		bytes -= (size_t)w;
		offset += (uint64_t)w;
	}
	return kOk;
}

AmpFileWriter::~AmpFileWriter()
{
	if (fd >= 0) {
		::close(fd);
		::unlink(tmp.c_str());
	}
}

int AmpFileWriter::create(const char* finalPath)
{
	path = finalPath;
	tmp = path + ".tmp";
	fd = ::open(tmp.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
	if (fd < 0)
		return setError(kErrIo, "cannot create '" + tmp + "': " + std::strerror(errno));
	return kOk;
}

int AmpFileWriter::commit()
{
	const int f = fd;
	fd = -1;
	if (::close(f) != 0) {
		::unlink(tmp.c_str());
		return setError(kErrIo, "close failed for '" + tmp + "'");
	}
	if (::rename(tmp.c_str(), path.c_str()) != 0) {
		const int e = errno;
		::unlink(tmp.c_str());
		return setError(kErrIo, "cannot rename '" + tmp + "' to '" + path + "': " + std::strerror(e));
	}
	return kOk;
}

}  // namespace pwa

extern "C" int pwa_ampfile_write(const char* path, uint32_t nWaves, const char* const* waveNames, uint64_t nEvents,
                                 const void* amps, uint32_t nVars, const char* const* varNames, const double* vars)
{
	if (!path || (nWaves && (!waveNames || !amps)) || (nVars && (!varNames || !vars)))
		return setError(kErrArg, "pwa_ampfile_write: null argument");
	if (nWaves == 0)
		return setError(kErrArg, "pwa_ampfile_write: no waves");
	std::vector<const char*> names(waveNames, waveNames + nWaves);
	names.insert(names.end(), varNames, varNames + nVars);
	std::vector<unsigned char> h;
	PWA_CHECK(ampFileHeader(nWaves, nVars, names.data(), nEvents, h));
	AmpFileWriter out;
	PWA_CHECK(out.create(path));
	PWA_CHECK(writeAll(out.fd, h.data(), h.size(), path));
	PWA_CHECK(writeAll(out.fd, amps, (size_t)(nEvents * 8ull * nWaves), path));
	if (nVars)
		PWA_CHECK(writeAll(out.fd, vars, (size_t)(nEvents * 8ull * nVars), path));
	return out.commit();
}

extern "C" int pwa_ampfile_info(const char* path, uint32_t* nWaves, uint64_t* nEvents, uint32_t* nVars)
{
	if (!path)
		return setError(kErrArg, "pwa_ampfile_info: null path");
	AmpFile f;
	const int st = ampFileOpen(path, f);
	if (st != kOk)
		return st;
	if (nWaves)
		*nWaves = f.nWaves;
	if (nEvents)
		*nEvents = f.nEvents;
	if (nVars)
		*nVars = f.nVars;
	return kOk;
}

extern "C" int pwa_ampfile_name(const char* path, int isVariable, uint32_t i, char* buf, uint32_t bufLen)
{
	if (!path || !buf || bufLen == 0)
		return setError(kErrArg, "pwa_ampfile_name: null argument");
	AmpFile f;
	const int st = ampFileOpen(path, f);
	if (st != kOk)
		return st;
	const std::vector<std::string>& v = isVariable ? f.vars : f.waves;
	if (i >= v.size())
		return setError(kErrArg, "pwa_ampfile_name: index out of range");
	if (v[i].size() + 1 > bufLen)
		return setError(kErrArg, "pwa_ampfile_name: buffer too small");
	std::memcpy(buf, v[i].c_str(), v[i].size() + 1);
	return kOk;
}
