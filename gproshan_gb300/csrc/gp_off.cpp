// OFF mesh reader: che_off::read_file (src/che_off.cpp:28-79).
//
// Token stream as the reference reads it: a header word (OFF, COFF or NOFF),
// the vertex, face and edge counts, then per vertex x y z (COFF: four colour
// values follow and are skipped; NOFF: three normal components), then per
// face a vertex count and the indices.  Triangles are kept; a quad a b c d
// becomes the triangles (a, b, c) and (d, a, c), the split the reference
// makes.  Unlike the reference this reader also skips '#' comments, accepts
// triangles and quads mixed in one file, and reports malformed input instead
// of reading past it.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gp_internal.h"

namespace {

struct Tok {
	const char *p, *end;

	bool skip()
	{
		for(;;)
		{
			while(p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
			if(p < end && *p == '#')
			{
				while(p < end && *p != '\n') p++;
				continue;
			}
			return p < end;
		}
	}

	bool word(std::string &w)
	{
		if(!skip()) return false;
		const char *q = p;
		while(p < end && !(*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
		w.assign(q, p);
		return true;
	}

	bool real(double &x)
	{
		if(!skip()) return false;
		char *e = nullptr;
		x = std::strtod(p, &e);
		if(e == p || e > end) return false;
		p = e;
		return true;
	}

	bool index(unsigned long &x)
	{
		if(!skip()) return false;
		char *e = nullptr;
		errno = 0;
		x = std::strtoul(p, &e, 10);
		if(e == p || e > end || errno) return false;
		p = e;
		return true;
	}
};

bool read_all(const char *path, std::vector<char> &buf)
{
	FILE *f = std::fopen(path, "rb");
	if(!f) return false;
	char chunk[1 << 16];
	size_t n;
	while((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
	const bool ok = !std::ferror(f);
	std::fclose(f);
	buf.push_back('\0');  // strtod/strtoul stop here at the latest
	return ok;
}

} // namespace

namespace gp {

// Parse an OFF file: xyz (3 per vertex) and triangles (3 per face, quads
// split).  Returns GP_OK, or GP_ERR_INVALID_ARG with a message in `err`.
gp_status off_parse(const char *path, std::vector<double> &xyz, std::vector<uint32_t> &tri, std::string &err)
{
	std::vector<char> buf;
	if(!path || !read_all(path, buf))
	{
		err = std::string("cannot read ") + (path ? path : "(null)");
		return GP_ERR_INVALID_ARG;
	}
	Tok t{buf.data(), buf.data() + buf.size() - 1};
	std::string head;
	if(!t.word(head) || (head != "OFF" && head != "COFF" && head != "NOFF"))
	{
		err = "not an OFF file (header '" + head + "')";
		return GP_ERR_INVALID_ARG;
	}
	unsigned long nv = 0, nf = 0, ne = 0;
	if(!t.index(nv) || !t.index(nf) || !t.index(ne) || nv >= 0x7FFFFFFFul || nf >= 0x2AAAAAAAul)
	{
		err = "bad OFF counts";
		return GP_ERR_INVALID_ARG;
	}
	const int extra = head[0] == 'C' ? 4 : head[0] == 'N' ? 3 : 0;
	xyz.resize(3 * nv);
	for(unsigned long v = 0; v < nv; v++)
	{
		for(int k = 0; k < 3; k++)
			if(!t.real(xyz[3 * v + k]))
			{
				err = "vertex " + std::to_string(v) + ": expected 3 coordinates";
				return GP_ERR_INVALID_ARG;
			}
		double skip;
		for(int k = 0; k < extra; k++)
			if(!t.real(skip))
			{
				err = "vertex " + std::to_string(v) + ": missing colour/normal values";
				return GP_ERR_INVALID_ARG;
			}
	}
	tri.clear();
	tri.reserve(3 * nf);
	for(unsigned long f = 0; f < nf; f++)
	{
		unsigned long k = 0, id[4];
		if(!t.index(k) || k < 3 || k > 4)
		{
			err = "face " + std::to_string(f) + ": only triangles and quads are supported";
			return GP_ERR_INVALID_ARG;
		}
		for(unsigned long q = 0; q < k; q++)
			if(!t.index(id[q]) || id[q] >= nv)
			{
				err = "face " + std::to_string(f) + ": bad vertex index";
				return GP_ERR_INVALID_ARG;
			}
		tri.push_back((uint32_t) id[0]);
		tri.push_back((uint32_t) id[1]);
		tri.push_back((uint32_t) id[2]);
		if(k == 4)
		{
			tri.push_back((uint32_t) id[3]);
			tri.push_back((uint32_t) id[0]);
			tri.push_back((uint32_t) id[2]);
		}
	}
	return GP_OK;
}

} // namespace gp
