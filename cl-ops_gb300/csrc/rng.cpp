// RNG objects: seed buffers for the four seed modes, the DEV_GID seed-hash
// compiler, host-side MT19937 seeding and the batched draw entry point.
// Reference behaviour: src/cl_ops/rng/clo_rng.c:60-483 and
// src/cl_ops/rng/clo_rng_init.cl:27-60.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "clo_internal.h"

using clo::cuda_ok;
using clo::set_error;

// Text of include/clo_rng_device.cuh, generated at build time.
#include "_gen_rng_device_src.inc"

struct clo_rng {
	int gen;
	std::string src;
	CCLBuffer *seeds_device;
	size_t size_in_device;
	size_t count;
};

extern "C" {
// Seed sizes as in the reference table (clo_rng.c:60-68); `src` is the
// macro that selects the generator in clo_rng_device.cuh.
const struct clo_rng_info clo_rng_infos[] = {
	{"lcg", "#define CLO_RNG_LCG\n", 8},
	{"xorshift64", "#define CLO_RNG_XORSHIFT64\n", 8},
	{"xorshift128", "#define CLO_RNG_XORSHIFT128\n", 16},
	{"mwc64x", "#define CLO_RNG_MWC64X\n", 8},
	{"parkmiller", "#define CLO_RNG_PARKMILLER\n", 4},
	{"tauslcg", "#define CLO_RNG_TAUSLCG\n", 16},
	{nullptr, nullptr, 0}};
}

namespace {

// ---------------------------------------------------------------------
// MT19937 (Matsumoto & Nishimura, 1998): init_genrand seeding and the
// tempered 32-bit output. GLib's GRand, which the reference's HOST_MT
// mode draws from (clo_rng.c:196-203), is this generator.
// ---------------------------------------------------------------------
struct Mt19937 {
	uint32_t mt[624];
	int mti;
	explicit Mt19937(uint32_t seed) {
		mt[0] = seed;
		for (mti = 1; mti < 624; mti++)
			mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) +
				(uint32_t)mti;
	}
	uint32_t next() {
		static const uint32_t mag01[2] = {0u, 0x9908b0dfu};
		if (mti >= 624) {
			int k;
			for (k = 0; k < 624 - 397; k++) {
				uint32_t y = (mt[k] & 0x80000000u) | (mt[k + 1] & 0x7fffffffu);
				mt[k] = mt[k + 397] ^ (y >> 1) ^ mag01[y & 1u];
			}
			for (; k < 623; k++) {
				uint32_t y = (mt[k] & 0x80000000u) | (mt[k + 1] & 0x7fffffffu);
				mt[k] = mt[k + (397 - 624)] ^ (y >> 1) ^ mag01[y & 1u];
			}
			uint32_t y = (mt[623] & 0x80000000u) | (mt[0] & 0x7fffffffu);
			mt[623] = mt[396] ^ (y >> 1) ^ mag01[y & 1u];
			mti = 0;
		}
		uint32_t y = mt[mti++];
		y ^= (y >> 11);
		y ^= (y << 7) & 0x9d2c5680u;
		y ^= (y << 15) & 0xefc60000u;
		y ^= (y >> 18);
		return y;
	}
};

// ---------------------------------------------------------------------
// DEV_GID seed hash. The reference pastes `hash` as the body of
// `#define CLO_RNG_HASH(x)` and applies it as a statement to the ulong
// seed (clo_rng.c:102-109, clo_rng_init.cl:55). This compiles the same
// text -- C statements over x with integer literals and the operators
// + - * / % & | ^ << >> ~ ! == != < > <= >= && || and compound
// assignments, plus the two predefined macros KNUTH(x) and XS1(x)
// (clo_rng_init.cl:27-33) -- into a stack program the init kernel runs.
// All arithmetic is on 64-bit unsigned values, as it is in the reference
// once x (a ulong) takes part; shift counts are masked to 6 bits as
// OpenCL does.
// ---------------------------------------------------------------------
enum HashOp : uint8_t {
	H_IMM, H_X, H_STORE, H_POP, H_ADD, H_SUB, H_MUL, H_DIV, H_MOD, H_AND,
	H_OR, H_XOR, H_SHL, H_SHR, H_NEG, H_NOT, H_LNOT, H_EQ, H_NE, H_LT, H_GT,
	H_LE, H_GE, H_LAND, H_LOR
};

struct HashCompiler {
	std::string s;
	size_t p = 0;
	clo::HashProgram prog{};
	std::string error;

	void emit(uint8_t op, uint64_t imm = 0) {
		if (prog.n_ops >= clo::HashProgram::MAX_OPS) {
			error = "hash program too long";
			return;
		}
		prog.op[prog.n_ops] = op;
		prog.imm[prog.n_ops] = imm;
		prog.n_ops++;
	}
	void ws() {
		while (p < s.size() && isspace((unsigned char)s[p])) p++;
	}
	bool eat(const char *t) {
		ws();
		size_t n = strlen(t);
		if (s.compare(p, n, t) == 0) {
			// Do not split a longer operator ("<" must not eat "<<").
			if (n == 1 && p + 1 < s.size()) {
				char a = s[p], b = s[p + 1];
				if ((a == '<' || a == '>') && (b == a || b == '=')) return false;
				if ((a == '&' && b == '&') || (a == '|' && b == '|')) return false;
				if ((a == '=' || a == '!') && b == '=') return false;
				if (strchr("+-*/%&|^", a) && b == '=') return false;
			}
			if (n == 2 && p + 2 < s.size() && (t[0] == '<' || t[0] == '>') &&
				t[1] == t[0] && s[p + 2] == '=')
				return false;
			p += n;
			return true;
		}
		return false;
	}
	bool is_ident_char(char c) { return isalnum((unsigned char)c) || c == '_'; }
	bool peek_x_assign(size_t &after, uint8_t &op) {
		ws();
		size_t q = p;
		if (q < s.size() && s[q] == 'x' && (q + 1 >= s.size() || !is_ident_char(s[q + 1]))) {
			q++;
			while (q < s.size() && isspace((unsigned char)s[q])) q++;
			static const struct { const char *t; uint8_t op; } ops[] = {
				{"<<=", H_SHL}, {">>=", H_SHR}, {"+=", H_ADD}, {"-=", H_SUB},
				{"*=", H_MUL}, {"/=", H_DIV}, {"%=", H_MOD}, {"&=", H_AND},
				{"|=", H_OR}, {"^=", H_XOR}};
			for (auto &o : ops) {
				size_t n = strlen(o.t);
				if (s.compare(q, n, o.t) == 0) {
					after = q + n;
					op = o.op;
					return true;
				}
			}
			if (q < s.size() && s[q] == '=' && (q + 1 >= s.size() || s[q + 1] != '=')) {
				after = q + 1;
				op = H_STORE;
				return true;
			}
		}
		return false;
	}
	bool number(uint64_t &v) {
		ws();
		if (p >= s.size() || !isdigit((unsigned char)s[p])) return false;
		const char *b = s.c_str() + p;
		char *e = nullptr;
		v = strtoull(b, &e, 0);  // decimal, 0x hex, leading-0 octal
		p += (size_t)(e - b);
		while (p < s.size() && strchr("uUlL", s[p])) p++;
		return true;
	}
	// Assignment expression: x op= expr is an expression whose value is
	// the new x.
	void assign_expr() {
		size_t after;
		uint8_t op;
		if (peek_x_assign(after, op)) {
			p = after;
			if (op == H_STORE) {
				assign_expr();
			} else {
				emit(H_X);
				assign_expr();
				emit(op);
			}
			emit(H_STORE);
			emit(H_X);
			return;
		}
		lor();
	}
	void lor() {
		land();
		while (error.empty() && eat("||")) { land(); emit(H_LOR); }
	}
	void land() {
		bor();
		while (error.empty() && eat("&&")) { bor(); emit(H_LAND); }
	}
	void bor() {
		bxor();
		while (error.empty() && eat("|")) { bxor(); emit(H_OR); }
	}
	void bxor() {
		band();
		while (error.empty() && eat("^")) { band(); emit(H_XOR); }
	}
	void band() {
		equality();
		while (error.empty() && eat("&")) { equality(); emit(H_AND); }
	}
	void equality() {
		relational();
		for (;;) {
			if (eat("==")) { relational(); emit(H_EQ); }
			else if (eat("!=")) { relational(); emit(H_NE); }
			else break;
		}
	}
	void relational() {
		shift();
		for (;;) {
			if (eat("<=")) { shift(); emit(H_LE); }
			else if (eat(">=")) { shift(); emit(H_GE); }
			else if (eat("<")) { shift(); emit(H_LT); }
			else if (eat(">")) { shift(); emit(H_GT); }
			else break;
		}
	}
	void shift() {
		additive();
		for (;;) {
			if (eat("<<")) { additive(); emit(H_SHL); }
			else if (eat(">>")) { additive(); emit(H_SHR); }
			else break;
		}
	}
	void additive() {
		mult();
		for (;;) {
			if (eat("+")) { mult(); emit(H_ADD); }
			else if (eat("-")) { mult(); emit(H_SUB); }
			else break;
		}
	}
	void mult() {
		unary();
		for (;;) {
			if (eat("*")) { unary(); emit(H_MUL); }
			else if (eat("/")) { unary(); emit(H_DIV); }
			else if (eat("%")) { unary(); emit(H_MOD); }
			else break;
		}
	}
	void unary() {
		if (eat("-")) { unary(); emit(H_NEG); return; }
		if (eat("+")) { unary(); return; }
		if (eat("~")) { unary(); emit(H_NOT); return; }
		if (eat("!")) { unary(); emit(H_LNOT); return; }
		primary();
	}
	void primary() {
		ws();
		uint64_t v;
		if (number(v)) {
			emit(H_IMM, v);
			return;
		}
		if (eat("(")) {
			// A cast to a 64-bit integer type is accepted and ignored: every
			// value is already 64-bit unsigned.
			static const char *casts[] = {"ulong", "long", "size_t"};
			for (const char *c : casts) {
				size_t n = strlen(c), q = p;
				while (q < s.size() && isspace((unsigned char)s[q])) q++;
				if (s.compare(q, n, c) == 0) {
					size_t r = q + n;
					while (r < s.size() && isspace((unsigned char)s[r])) r++;
					if (r < s.size() && s[r] == ')') {
						p = r + 1;
						unary();
						return;
					}
				}
			}
			assign_expr();
			if (!eat(")")) error = "expected ')'";
			return;
		}
		if (p < s.size() && s[p] == 'x' &&
			(p + 1 >= s.size() || !is_ident_char(s[p + 1]))) {
			p++;
			emit(H_X);
			return;
		}
		error = "unexpected token at '" + s.substr(p, 16) + "'";
	}
	bool compile(const std::string &text) {
		// Expand the two predefined hashes of clo_rng_init.cl:27-33.
		std::string t = text;
		auto expand = [&](const char *name, const char *body) {
			for (;;) {
				size_t k = t.find(name);
				if (k == std::string::npos) break;
				size_t q = k + strlen(name);
				while (q < t.size() && isspace((unsigned char)t[q])) q++;
				if (q >= t.size() || t[q] != '(') break;
				size_t r = t.find(')', q);
				if (r == std::string::npos) break;
				std::string arg = t.substr(q + 1, r - q - 1);
				std::string a2;
				for (char c : arg)
					if (!isspace((unsigned char)c)) a2 += c;
				if (a2 != "x") {
					error = std::string(name) + " takes the seed variable x";
					return;
				}
				t = t.substr(0, k) + body + t.substr(r + 1);
			}
		};
		expand("KNUTH", "x = ((x*2654435761) % 0x100000000)");
		expand("XS1", "x = ((x >> 16) ^ x) * 0x45d9f3b; "
			"x = ((x >> 16) ^ x) * 0x45d9f3b; x = ((x >> 16) ^ x);");
		if (!error.empty()) return false;
		s = t;
		p = 0;
		prog.n_ops = 0;
		for (;;) {
			ws();
			if (p >= s.size()) break;
			if (s[p] == ';') {
				p++;
				continue;
			}
			assign_expr();
			if (!error.empty()) return false;
			emit(H_POP);
			ws();
			if (p < s.size() && s[p] != ';') {
				error = "expected ';' at '" + s.substr(p, 16) + "'";
				return false;
			}
		}
		if (!error.empty()) return false;
		// The device interpreter keeps a 16-entry stack.
		int depth = 0, maxd = 0;
		for (int i = 0; i < prog.n_ops; ++i) {
			uint8_t o = prog.op[i];
			if (o == H_IMM || o == H_X) depth++;
			else if (o == H_STORE || o == H_POP) depth--;
			else if (o == H_NEG || o == H_NOT || o == H_LNOT) {}
			else depth--;
			if (depth > maxd) maxd = depth;
			if (depth < 0) { error = "malformed hash"; return false; }
		}
		if (maxd > 16) { error = "hash expression nested too deeply"; return false; }
		return true;
	}
};

size_t seed_size(int gen) { return clo_rng_infos[gen].seed_size; }

}  // namespace

namespace clo {
// Host reference of the hash stack program, used to validate programs.
bool hash_compile(const char *text, HashProgram &out, std::string &error) {
	HashCompiler c;
	std::string t = (text && *text) ? text : "x";
	if (!c.compile(t)) {
		error = c.error;
		return false;
	}
	out = c.prog;
	return true;
}
}  // namespace clo

extern "C" {

CloRng *clo_rng_new(const char *type, CloRngSeedType seed_type, void *seeds,
	size_t seeds_count, cl_ulong main_seed, const char *hash, CCLContext *ctx,
	CCLQueue *cq, GError **err) {
	if (err && *err) return nullptr;
	int gen = -1;
	for (int i = 0; clo_rng_infos[i].name; ++i)
		if (type && strcmp(type, clo_rng_infos[i].name) == 0) gen = i;
	if (gen < 0) {
		set_error(err, CLO_ERROR_IMPL_NOT_FOUND,
			"The requested RNG implementation, '%s', was not found.",
			type ? type : "(null)");
		return nullptr;
	}
	if (!ctx || !cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL context or queue");
		return nullptr;
	}
	cudaSetDevice(ctx->ordinal);
	size_t bytes = seeds_count * seed_size(gen);
	CCLBuffer *dev = nullptr;
	switch (seed_type) {
	case CLO_RNG_SEED_DEV_GID: {
		if (seeds != nullptr) {
			set_error(err, CLO_ERROR_ARGS,
				"The DEV_GID seed type expects a NULL seeds parameter.");
			return nullptr;
		}
		clo::HashProgram hp;
		std::string msg;
		if (!clo::hash_compile(hash, hp, msg)) {
			set_error(err, CLO_ERROR_ARGS, "Invalid seed hash '%s': %s",
				hash ? hash : "", msg.c_str());
			return nullptr;
		}
		dev = ccl_buffer_new(ctx, CL_MEM_READ_WRITE, bytes, nullptr, err);
		if (!dev) return nullptr;
		if (!cuda_ok(clo::rng_init_gid(dev->ptr, seeds_count, gen, main_seed,
				hp, cq->stream), err, "clo_rng_init")) {
			ccl_buffer_destroy(dev);
			return nullptr;
		}
		break;
	}
	case CLO_RNG_SEED_HOST_MT: {
		if (seeds != nullptr) {
			set_error(err, CLO_ERROR_ARGS,
				"The HOST_MT seed type expects a NULL seeds parameter.");
			return nullptr;
		}
		std::vector<uint32_t> words(bytes / 4 + 1);
		Mt19937 mt((uint32_t)main_seed);
		for (size_t i = 0; i < bytes / 4; ++i) words[i] = mt.next();
		dev = ccl_buffer_new(ctx, CL_MEM_READ_WRITE, bytes, nullptr, err);
		if (!dev) return nullptr;
		if (bytes && !cuda_ok(cudaMemcpyAsync(dev->ptr, words.data(), bytes,
				cudaMemcpyHostToDevice, cq->stream), err, "seed write")) {
			ccl_buffer_destroy(dev);
			return nullptr;
		}
		cudaStreamSynchronize(cq->stream);
		break;
	}
	case CLO_RNG_SEED_EXT_DEV: {
		CCLBuffer *ext = (CCLBuffer *)seeds;
		if (!ext || ext->size < bytes) {
			set_error(err, CLO_ERROR_ARGS,
				"The '%s' RNG type requires a buffer of at least %zu bytes. The "
				"size of the provided external device seeds buffer is only %zu "
				"bytes.", type, bytes, ext ? ext->size : (size_t)0);
			return nullptr;
		}
		ccl_buffer_ref(ext);
		dev = ext;
		break;
	}
	case CLO_RNG_SEED_EXT_HOST: {
		if (seeds == nullptr) {
			set_error(err, CLO_ERROR_ARGS,
				"The EXT_HOST seed type expects a non-NULL seeds parameter.");
			return nullptr;
		}
		dev = ccl_buffer_new(ctx, CL_MEM_READ_WRITE, bytes, nullptr, err);
		if (!dev) return nullptr;
		if (bytes && !cuda_ok(cudaMemcpyAsync(dev->ptr, seeds, bytes,
				cudaMemcpyHostToDevice, cq->stream), err, "seed write")) {
			ccl_buffer_destroy(dev);
			return nullptr;
		}
		cudaStreamSynchronize(cq->stream);
		break;
	}
	default:
		set_error(err, CLO_ERROR_ARGS, "Unknown seed type.");
		return nullptr;
	}
	CloRng *rng = new clo_rng();
	rng->gen = gen;
	rng->src = std::string(clo_rng_infos[gen].src) + kRngDeviceSource;
	rng->seeds_device = dev;
	rng->size_in_device = bytes;
	rng->count = seeds_count;
	return rng;
}

void clo_rng_destroy(CloRng *rng) {
	if (!rng) return;
	ccl_buffer_destroy(rng->seeds_device);
	delete rng;
}

const char *clo_rng_get_source(CloRng *rng) {
	return rng ? rng->src.c_str() : nullptr;
}

CCLBuffer *clo_rng_get_device_seeds(CloRng *rng) {
	return rng ? rng->seeds_device : nullptr;
}

size_t clo_rng_get_size(CloRng *rng) { return rng ? rng->size_in_device : 0; }

CCLEvent *clo_rng_fill(CloRng *rng, CCLQueue *cq, CCLBuffer *out,
	size_t draws, cl_uint bits, cl_uint maxint, GError **err) {
	if (!rng || !cq || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_rng_fill: bad arguments\n");
		return nullptr;
	}
	if (maxint == 0 && (bits < 1 || bits > 32)) {
		set_error(err, CLO_ERROR_ARGS,
			"Number of bits must be between 1 and 32.");
		return nullptr;
	}
	if (!out || out->size < draws * rng->count * sizeof(uint32_t)) {
		set_error(err, CLO_ERROR_ARGS,
			"Output buffer must hold %zu x %zu uint values", draws, rng->count);
		return nullptr;
	}
	cudaSetDevice(cq->ctx->ordinal);
	ccl_event *ev = clo::event_begin(cq, "clo_rng_fill");
	if (!cuda_ok(clo::rng_fill(rng->seeds_device->ptr, rng->count, rng->gen,
			(uint32_t *)out->ptr, draws, bits, maxint, cq->stream), err,
			"clo_rng_fill"))
		return nullptr;
	clo::event_end(ev);
	return ev;
}

}  // extern "C"
