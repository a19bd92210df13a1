// wire.cpp — circuit wire formats: the QASM3 subset the reference imports
// (butterfly/utils/qasm3_import.mojo:1-123) and a self-contained binary
// op list for handing circuits across a process or network boundary (the
// serve API).  Both produce an owned op list (bf_oplist): bf_op records whose
// data / qubits pointers refer to storage inside the list.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bf_internal.h"

namespace bf {

struct OpList {
  int32_t num_qubits = 0;
  std::vector<bf_op> ops;
  std::vector<std::vector<double>> data;
  std::vector<std::vector<int32_t>> qubits;

  // re-points every op at this list's own storage
  void bind() {
    for (size_t i = 0; i < ops.size(); ++i) {
      ops[i].data = data[i].empty() ? nullptr : data[i].data();
      ops[i].qubits = qubits[i].empty() ? nullptr : qubits[i].data();
    }
  }
  void push(const bf_op& o, std::vector<double> d = {}, std::vector<int32_t> q = {}) {
    ops.push_back(o);
    data.push_back(std::move(d));
    qubits.push_back(std::move(q));
  }
};

// doubles an op's data pointer refers to
size_t op_data_len(const bf_op& o) {
  switch (o.kind) {
    case BF_OP_UNITARY:
    case BF_OP_CUNITARY:
      return (o.target2 > 0 && o.target2 < 16) ? 2 * ((size_t)1 << (2 * o.target2)) : 0;
    case BF_OP_MEASURE:
    case BF_OP_CLASSICAL_ORACLE:
    case BF_OP_MODEXP:
    case BF_OP_MODEXP_INV:
      return (size_t)std::max<int64_t>(0, o.nqubits);
    default:
      return 0;
  }
}

// int32 entries an op's qubits pointer refers to
size_t op_qubits_len(const bf_op& o) {
  switch (o.kind) {
    case BF_OP_QREV:
    case BF_OP_BITREV:
    case BF_OP_PERMUTE:
    case BF_OP_MEASURE:
    case BF_OP_GROVER_DIFFUSER:
    case BF_OP_GROVER_INVERSION0:
      return (size_t)std::max<int64_t>(0, o.nqubits);
    default:
      return 0;
  }
}

// ---- QASM3 subset ---------------------------------------------------------------
// Lines: blank, "//" comments, OPENQASM, include, "qubit[n] q;", then
// "h q[i];", "x q[i];", "p(angle) q[i];", "cp(angle) q[c], q[t];".  Angles:
// a number, pi, -pi, k*pi, pi/k, k/pi (parse_angle, qasm3_import.mojo:7-30).
namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

double parse_number(const std::string& t, const std::string& line) {
  std::string s = trim(t);
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  if (s.empty() || end != s.c_str() + s.size()) fail(BF_EINVAL, "Invalid number in QASM: %s", line.c_str());
  return v;
}

double parse_angle(const std::string& expr, const std::string& line) {
  std::string s = trim(expr);
  if (s.find("pi") != std::string::npos) {
    std::string t;
    for (char c : s)
      if (c != ' ') t += c;
    double sign = 1.0;
    if (!t.empty() && t[0] == '-') {
      sign = -1.0;
      t = t.substr(1);
    }
    const double pi = 3.141592653589793;
    if (t == "pi") return sign * pi;
    if (t.size() > 3 && t.compare(t.size() - 3, 3, "*pi") == 0)
      return sign * parse_number(t.substr(0, t.size() - 3), line) * pi;
    if (t.compare(0, 3, "pi/") == 0) return sign * pi / parse_number(t.substr(3), line);
    size_t k = t.find("/pi");
    if (k != std::string::npos && k + 3 == t.size()) return sign * parse_number(t.substr(0, k), line) / pi;
  }
  return parse_number(s, line);
}

// an integer in [lo, hi] (checked before any conversion to int)
int parse_int(const std::string& t, const std::string& line, int lo, int hi) {
  const double v = parse_number(t, line);
  if (!(v >= lo && v <= hi) || v != std::floor(v)) fail(BF_EINVAL, "Integer out of range in QASM: %s", line.c_str());
  return (int)v;
}

// "q[3]" (optionally followed by ';' or ',') -> 3
int parse_qubit(const std::string& token) {
  std::string t = trim(token);
  if (!t.empty() && t.back() == ';') t = trim(t.substr(0, t.size() - 1));
  if (!t.empty() && t.back() == ',') t = trim(t.substr(0, t.size() - 1));
  size_t lb = t.find('['), rb = t.find(']');
  if (lb == std::string::npos || rb == std::string::npos || rb <= lb) fail(BF_EINVAL, "Invalid qubit token: %s", t.c_str());
  return parse_int(t.substr(lb + 1, rb - lb - 1), t, 0, 63);
}

bf_op gate_op(int gate, int target, double arg) {
  bf_op o;
  std::memset(&o, 0, sizeof o);
  o.kind = BF_OP_GATE;
  o.gate = gate;
  o.target = target;
  o.arg = arg;
  return o;
}

}  // namespace

OpList* qasm3_parse(const char* text) {
  if (!text) fail(BF_EINVAL, "QASM text is null");
  auto* L = new OpList();
  try {
    bool has = false;
    std::string all(text);
    size_t pos = 0;
    while (pos <= all.size()) {
      size_t nl = all.find('\n', pos);
      if (nl == std::string::npos) nl = all.size();
      std::string s = trim(all.substr(pos, nl - pos));
      pos = nl + 1;
      if (s.empty() || s.compare(0, 2, "//") == 0 || s.compare(0, 8, "OPENQASM") == 0 || s.compare(0, 7, "include") == 0)
        continue;
      if (s.compare(0, 5, "qubit") == 0) {
        size_t lb = s.find('['), rb = s.find(']');
        if (lb == std::string::npos || rb == std::string::npos || rb <= lb)
          fail(BF_EINVAL, "Invalid qubit declaration: %s", s.c_str());
        L->num_qubits = parse_int(s.substr(lb + 1, rb - lb - 1), s, 1, 64);
        L->ops.clear();
        L->data.clear();
        L->qubits.clear();
        has = true;
        continue;
      }
      if (!has) fail(BF_EINVAL, "QASM missing qubit declaration before gates.");
      if (!s.empty() && s.back() == ';') s = trim(s.substr(0, s.size() - 1));
      if (s.compare(0, 2, "h ") == 0) {
        L->push(gate_op(BF_GATE_H, parse_qubit(s.substr(2)), 0.0));
      } else if (s.compare(0, 2, "x ") == 0) {
        L->push(gate_op(BF_GATE_X, parse_qubit(s.substr(2)), 0.0));
      } else if (s.compare(0, 2, "p(") == 0) {
        size_t close = s.find(')');
        if (close == std::string::npos) fail(BF_EINVAL, "Invalid p gate: %s", s.c_str());
        L->push(gate_op(BF_GATE_P, parse_qubit(s.substr(close + 1)), parse_angle(s.substr(2, close - 2), s)));
      } else if (s.compare(0, 3, "cp(") == 0) {
        size_t close = s.find(')');
        if (close == std::string::npos) fail(BF_EINVAL, "Invalid cp gate: %s", s.c_str());
        std::string rest = trim(s.substr(close + 1));
        size_t comma = rest.find(',');
        if (comma == std::string::npos || rest.find(',', comma + 1) != std::string::npos)
          fail(BF_EINVAL, "Invalid cp operands: %s", rest.c_str());
        int c = parse_qubit(rest.substr(0, comma)), t = parse_qubit(rest.substr(comma + 1));
        bf_op o = gate_op(BF_GATE_P, t, parse_angle(s.substr(3, close - 3), s));
        if (c < 0 || c >= 64) fail(BF_EINVAL, "Control out of bounds: %d", c);
        o.controls = 1ull << c;
        o.ncontrols = 1;
        L->push(o);
      } else {
        fail(BF_EINVAL, "Unsupported QASM line: %s", s.c_str());
      }
    }
    if (!has) fail(BF_EINVAL, "No qubit declaration found in QASM.");
    L->bind();
    return L;
  } catch (...) {
    delete L;
    throw;
  }
}

// ---- binary op list -----------------------------------------------------------
// Little-endian.  Header: "BFOP", u32 version (1), i32 num_qubits,
// u32 reserved, i64 nops.  Each op: the 104 fixed bytes of bf_op (kind ..
// mat[8]), i64 nqubits, i64 data count, i64 qubit count, then the doubles,
// then the int32 qubits padded to 8 bytes.
namespace {
constexpr uint32_t kWireVersion = 1;
constexpr size_t kFixed = offsetof(bf_op, data);
static_assert(kFixed == 104, "bf_op fixed part");

void put(std::vector<unsigned char>& out, const void* p, size_t n) {
  const auto* b = static_cast<const unsigned char*>(p);
  out.insert(out.end(), b, b + n);
}
}  // namespace

std::vector<unsigned char> ops_serialize(int32_t n, const bf_op* ops, int64_t nops) {
  if (nops < 0 || (nops > 0 && !ops)) fail(BF_EINVAL, "ops is null");
  std::vector<unsigned char> out;
  put(out, "BFOP", 4);
  uint32_t ver = kWireVersion, res = 0;
  put(out, &ver, 4);
  put(out, &n, 4);
  put(out, &res, 4);
  put(out, &nops, 8);
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& o = ops[i];
    put(out, &o, kFixed);
    put(out, &o.nqubits, 8);
    int64_t nd = o.data ? (int64_t)op_data_len(o) : 0, nq = o.qubits ? (int64_t)op_qubits_len(o) : 0;
    put(out, &nd, 8);
    put(out, &nq, 8);
    if (nd) put(out, o.data, (size_t)nd * sizeof(double));
    if (nq) put(out, o.qubits, (size_t)nq * sizeof(int32_t));
    if (nq & 1) {
      int32_t pad = 0;
      put(out, &pad, 4);
    }
  }
  return out;
}

OpList* ops_deserialize(const void* blob, size_t len) {
  if (!blob) fail(BF_EINVAL, "blob is null");
  const auto* p = static_cast<const unsigned char*>(blob);
  size_t at = 0;
  auto take = [&](void* dst, size_t n) {
    if (n > len - at) fail(BF_EINVAL, "op list truncated at byte %zu", at);
    std::memcpy(dst, p + at, n);
    at += n;
  };
  if (len < 24 || std::memcmp(p, "BFOP", 4) != 0) fail(BF_EINVAL, "not a bfgpu op list");
  at = 4;
  uint32_t ver = 0, res = 0;
  int64_t nops = 0;
  auto* L = new OpList();
  try {
    take(&ver, 4);
    if (ver != kWireVersion) fail(BF_EINVAL, "op list version %u (expected %u)", ver, kWireVersion);
    take(&L->num_qubits, 4);
    if (L->num_qubits < 1 || L->num_qubits > 64)
      fail(BF_EINVAL, "op list qubit count %d is out of range", (int)L->num_qubits);
    take(&res, 4);
    take(&nops, 8);
    if (nops < 0 || (uint64_t)nops > (len - at) / (kFixed + 24)) fail(BF_EINVAL, "op list count %lld is invalid", (long long)nops);
    L->ops.reserve((size_t)nops);
    for (int64_t i = 0; i < nops; ++i) {
      bf_op o;
      std::memset(&o, 0, sizeof o);
      take(&o, kFixed);
      take(&o.nqubits, 8);
      int64_t nd = 0, nq = 0;
      take(&nd, 8);
      take(&nq, 8);
      if (nd < 0 || nq < 0 || (uint64_t)nd > (len - at) / 8 || (uint64_t)nq > (len - at) / 4)
        fail(BF_EINVAL, "op %lld has invalid lengths", (long long)i);
      std::vector<double> d((size_t)nd);
      std::vector<int32_t> q((size_t)nq);
      if (nd) take(d.data(), (size_t)nd * 8);
      if (nq) take(q.data(), (size_t)nq * 4);
      if (nq & 1) {
        int32_t pad;
        take(&pad, 4);
      }
      // the pointers of a record are restored only where their lengths agree
      if ((size_t)nd != 0 && (size_t)nd != op_data_len(o)) fail(BF_EINVAL, "op %lld: data length %lld does not match its kind", (long long)i, (long long)nd);
      if ((size_t)nq != 0 && (size_t)nq != op_qubits_len(o)) fail(BF_EINVAL, "op %lld: qubit count %lld does not match its kind", (long long)i, (long long)nq);
      L->push(o, std::move(d), std::move(q));
    }
    if (at != len) fail(BF_EINVAL, "op list has %zu trailing bytes", len - at);
    L->bind();
    return L;
  } catch (...) {
    delete L;
    throw;
  }
}

void oplist_view(const OpList& L, const bf_op** ops, int64_t* nops, int32_t* n) {
  if (ops) *ops = L.ops.empty() ? nullptr : L.ops.data();
  if (nops) *nops = (int64_t)L.ops.size();
  if (n) *n = L.num_qubits;
}

void oplist_destroy(OpList* L) { delete L; }

}  // namespace bf
