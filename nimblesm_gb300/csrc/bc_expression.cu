// Boundary-condition expressions f(x, y, z, t): the reference's grammar
// (src/nimble_expression_parser.h:522-695, src/nimble_expression_parser.cc:
// 45-190) restated as a parser to postfix programs that the node kernels
// evaluate per node.  The tree it builds is the reference's, operator by
// operator, so the arithmetic order (and with it the rounding) is the same:
//   * formatting: surrounding blanks and redundant outer parentheses are
//     dropped; the text is lower-cased once;
//   * a constant ("e", "pi", "tau", or a number: optional sign, digits, one
//     '.', an 'e' followed by an integer) ends the descent;
//   * operations are tried in this order, each split at depth 0 outside
//     parentheses: "c ? a : b" (first '?'), the LAST '%', the LAST '+', the
//     last '-' that is a binary minus (not after * / ^ e = < ~ >, not a
//     leading negation; split at the first '-' of a run), the LAST '*', the
//     LAST '/', then the FIRST '^' (an integer exponent text gives the integer
//     power), then a leading '-' (negation);
//   * then a function call name(arg) of the reference's list, then x, y, z, t;
//   * conditions: "true", "false", the last '|', '^' (xor), '&', a leading
//     '!', the last '>' / '>=', '<' / '<=', "==".
// Subtrees whose inputs are all constants are folded when parsed, with the
// host's <cmath>, as the reference's optimize() does; the device evaluates
// what remains with CUDA's double-precision functions.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "nsm_kernels.cuh"

namespace nsm {
namespace {

struct Node {
  int    code = kExConst;
  double c    = 0.0;
  int    in[3] = {-1, -1, -1};
};

bool is_digit(char c) { return c >= '0' && c <= '9'; }

bool is_integer(const std::string& s)
{
  if (s.empty()) return false;
  if (s.size() == 1 && (s[0] == '-' || s[0] == '+')) return false;
  if (s[0] != '-' && s[0] != '+' && !is_digit(s[0])) return false;
  for (size_t i = 1; i < s.size(); i++)
    if (!is_digit(s[i])) return false;
  return true;
}

bool is_number(const std::string& s)
{
  if (s.empty()) return false;
  size_t i       = (s[0] == '-' || s[0] == '+') ? 1 : 0;
  bool   decimal = false, digits = false;
  for (; i < s.size(); i++) {
    const char c = s[i];
    if (is_digit(c)) {
      digits = true;
    } else if (c == '.' && !decimal) {
      decimal = true;
    } else if (c == 'e' && digits) {
      return is_integer(s.substr(i + 1));
    } else {
      return false;
    }
  }
  return true;
}

// Blanks at both ends and parentheses that enclose everything.
std::string format(std::string s)
{
  size_t a = s.find_first_not_of(' ');
  if (a == std::string::npos) return std::string();
  size_t b = s.find_last_not_of(' ');
  s        = s.substr(a, b - a + 1);
  while (s.size() >= 2 && s[0] == '(') {
    int    depth = 0;
    size_t close = std::string::npos;
    for (size_t i = 0; i < s.size(); i++) {
      if (s[i] == '(') depth++;
      if (s[i] == ')' && --depth == 0) {
        close = i;
        break;
      }
    }
    if (close != s.size() - 1) break;
    s = s.substr(1, s.size() - 2);
  }
  return s;
}

// Position of the first (last) occurrence of c at parenthesis depth 0, or npos.
size_t first_at_depth0(const std::string& s, char c)
{
  int depth = 0;
  for (size_t i = 0; i < s.size(); i++) {
    if (depth == 0 && s[i] == c) return i;
    if (s[i] == '(') depth++;
    if (s[i] == ')') depth--;
  }
  return std::string::npos;
}
size_t last_at_depth0(const std::string& s, char c)
{
  int depth = 0;
  for (size_t i = s.size(); i-- > 0;) {
    if (depth == 0 && s[i] == c) return i;
    if (s[i] == ')') depth++;
    if (s[i] == '(') depth--;
  }
  return std::string::npos;
}

const char* const kFunctions[] = {"sin",  "cos",  "tan",  "erf",  "exp",  "log",   "abs",   "asin",  "acos",
                                  "atan", "sqrt", "cbrt", "erfc", "ceil", "round", "floor", "log10"};
const int kFunctionCodes[] = {kExSin,  kExCos,  kExTan,  kExErf,  kExExp,   kExLog,   kExAbs,  kExAsin, kExAcos,
                              kExAtan, kExSqrt, kExCbrt, kExErfc, kExCeil, kExRound, kExFloor, kExLog10};

class Parser {
 public:
  std::vector<Node> nodes;

  int equation(const std::string& text)
  {
    const std::string s = format(text);
    if (s.empty()) throw std::invalid_argument("can't parse an empty expression");
    if (s == "e") return constant(M_E);
    if (s == "pi") return constant(M_PI);
    if (s == "tau") return constant(M_PI * 2);
    if (is_number(s)) return constant(std::stod(s));
    int r = operation(s);
    if (r >= 0) return r;
    r = function(s);
    if (r >= 0) return r;
    if (s == "x") return leaf(kExX);
    if (s == "y") return leaf(kExY);
    if (s == "z") return leaf(kExZ);
    if (s == "t") return leaf(kExT);
    throw std::invalid_argument("unable to parse \"" + s + "\"");
  }

 private:
  int constant(double v)
  {
    Node n;
    n.code = kExConst;
    n.c    = v;
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  int leaf(int code)
  {
    Node n;
    n.code = code;
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  bool is_const(int i) const { return nodes[i].code == kExConst; }

  // A node of `code` over inputs; folded to a constant when they all are.
  int op(int code, int a, int b = -1, int c = -1)
  {
    Node n;
    n.code  = code;
    n.in[0] = a;
    n.in[1] = b;
    n.in[2] = c;
    if (code == kExSelect && is_const(a)) return nodes[a].c != 0.0 ? b : c;
    bool all = is_const(a) && (b < 0 || is_const(b)) && (c < 0 || is_const(c));
    if (all) {
      const double x = nodes[a].c, y = b >= 0 ? nodes[b].c : 0.0;
      return constant(apply_host(code, x, y));
    }
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }

  int operation(const std::string& s)
  {
    size_t q = first_at_depth0(s, '?');
    if (q != std::string::npos) {
      int    depth = 1;
      size_t k     = q;
      while (depth != 0 && k + 1 < s.size()) {
        const char c = s[++k];
        if (c == '?') depth++;
        if (c == ':') depth--;
      }
      if (depth > 0) throw std::invalid_argument("couldn't find the matching : of a ternary operator in " + s);
      return op(kExSelect, condition(s.substr(0, q)), equation(s.substr(q + 1, k - q - 1)),
                equation(s.substr(k + 1)));
    }
    size_t p = last_at_depth0(s, '%');
    if (p != std::string::npos) return op(kExMod, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    p = last_at_depth0(s, '+');
    if (p != std::string::npos) return op(kExAdd, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    p = last_at_depth0(s, '-');
    if (p != std::string::npos) {
      // back over the run of '-' and blanks; a binary minus has an operand
      // before it that does not end in an operator or an exponent's 'e'
      size_t k = p;
      while (k > 0 && (s[k] == '-' || s[k] == ' ')) k--;
      if (k > 0 || s[k] != '-') {
        const char c = s[k];
        if (c != '*' && c != '/' && c != '^' && c != 'e' && c != '=' && c != '<' && c != '~' && c != '>') {
          while (s[k] != '-') k++;
          return op(kExSub, equation(s.substr(0, k)), equation(s.substr(k + 1)));
        }
      }
    }
    p = last_at_depth0(s, '*');
    if (p != std::string::npos) return op(kExMul, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    p = last_at_depth0(s, '/');
    if (p != std::string::npos) return op(kExDiv, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    p = first_at_depth0(s, '^');
    if (p != std::string::npos) {
      const int         base  = equation(s.substr(0, p));
      const std::string power = format(s.substr(p + 1));
      if (is_integer(power)) return op(kExPow, base, constant((double)std::strtol(power.c_str(), nullptr, 10)));
      return op(kExPow, base, equation(power));
    }
    if (s[0] == '-') return op(kExNeg, equation(s.substr(1)));
    return -1;
  }

  int function(const std::string& s)
  {
    const char c0 = s[0];
    if (is_digit(c0) || c0 == '(' || c0 == '-' || s.size() < 3) return -1;
    size_t k = 0;
    while (k < s.size() && s[k] != '(' && s[k] != ' ') {
      const char c = s[k];
      if (c == '*' || c == '/' || c == '^' || c == '+' || c == '=' || c == '<' || c == '~' || c == '>') return -1;
      k++;
    }
    const size_t open = first_at_depth0(s, '(');
    if (open == std::string::npos) return -1;
    int    depth = 0;
    size_t close = std::string::npos;
    for (size_t i = open; i < s.size(); i++) {
      if (s[i] == '(') depth++;
      if (s[i] == ')' && --depth == 0) {
        close = i;
        break;
      }
    }
    if (close == std::string::npos) throw std::invalid_argument("mismatched parenthesis in " + s);
    if (close < s.size() - 1) return -1;
    const std::string name = s.substr(0, open);
    for (size_t f = 0; f < sizeof(kFunctions) / sizeof(kFunctions[0]); f++)
      if (name == kFunctions[f]) return op(kFunctionCodes[f], equation(s.substr(open)));
    return -1;
  }

  int condition(const std::string& text)
  {
    const std::string s = format(text);
    if (s == "true") return constant(1.0);
    if (s == "false") return constant(0.0);
    if (s.empty()) throw std::invalid_argument("unable to parse an empty condition");
    size_t p = last_at_depth0(s, '|');
    if (p != std::string::npos) return op(kExOr, condition(s.substr(0, p)), condition(s.substr(p + 1)));
    p = last_at_depth0(s, '^');
    if (p != std::string::npos) return op(kExXor, condition(s.substr(0, p)), condition(s.substr(p + 1)));
    p = last_at_depth0(s, '&');
    if (p != std::string::npos) return op(kExAnd, condition(s.substr(0, p)), condition(s.substr(p + 1)));
    if (s[0] == '!') return op(kExNot, condition(s.substr(1)));
    p = last_at_depth0(s, '>');
    if (p != std::string::npos) {
      if (p + 1 < s.size() && s[p + 1] == '=')
        return op(kExGe, equation(s.substr(0, p)), equation(s.substr(p + 2)));
      return op(kExGt, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    }
    p = last_at_depth0(s, '<');
    if (p != std::string::npos) {
      if (p + 1 < s.size() && s[p + 1] == '=')
        return op(kExLe, equation(s.substr(0, p)), equation(s.substr(p + 2)));
      return op(kExLt, equation(s.substr(0, p)), equation(s.substr(p + 1)));
    }
    p = last_at_depth0(s, '=');
    if (p != std::string::npos && p > 0 && s[p - 1] == '=')
      return op(kExEq, equation(s.substr(p + 1)), equation(s.substr(0, p - 1)));
    throw std::invalid_argument("unable to parse \"" + s + "\" as a condition");
  }

 public:
  // Postfix order of the tree under `root`; the stack depth it needs.
  int emit(int root, std::vector<ExprOp>& out) const
  {
    const Node& n = nodes[root];
    if (n.code == kExSelect) {
      const int d0 = emit(n.in[0], out);
      const int d1 = emit(n.in[1], out);
      const int d2 = emit(n.in[2], out);
      out.push_back(ExprOp{n.code, 0, 0.0});
      return std::max(d0, std::max(1 + d1, 2 + d2));
    }
    if (n.in[0] < 0) {
      out.push_back(ExprOp{n.code, 0, n.c});
      return 1;
    }
    const int d0 = emit(n.in[0], out);
    if (n.in[1] < 0) {
      out.push_back(ExprOp{n.code, 0, 0.0});
      return d0;
    }
    const int d1 = emit(n.in[1], out);
    out.push_back(ExprOp{n.code, 0, 0.0});
    return std::max(d0, 1 + d1);
  }
};

}  // namespace

// One operation on the host (constant folding and host evaluation).
double apply_host(int code, double a, double b)
{
  switch (code) {
    case kExAdd: return a + b;
    case kExSub: return a - b;
    case kExMul: return a * b;
    case kExDiv: return a / b;
    case kExMod: return std::fmod(a, b);
    case kExPow: return std::pow(a, b);
    case kExNeg: return -a;
    case kExSin: return std::sin(a);
    case kExCos: return std::cos(a);
    case kExTan: return std::tan(a);
    case kExErf: return std::erf(a);
    case kExExp: return std::exp(a);
    case kExLog: return std::log(a);
    case kExAbs: return std::fabs(a);
    case kExAsin: return std::asin(a);
    case kExAcos: return std::acos(a);
    case kExAtan: return std::atan(a);
    case kExSqrt: return std::sqrt(a);
    case kExCbrt: return std::cbrt(a);
    case kExErfc: return std::erfc(a);
    case kExCeil: return std::ceil(a);
    case kExRound: return std::round(a);
    case kExFloor: return std::floor(a);
    case kExLog10: return std::log10(a);
    case kExGt: return a > b ? 1.0 : 0.0;
    case kExGe: return a >= b ? 1.0 : 0.0;
    case kExLt: return a < b ? 1.0 : 0.0;
    case kExLe: return a <= b ? 1.0 : 0.0;
    case kExEq: return a == b ? 1.0 : 0.0;
    case kExAnd: return (a != 0.0 && b != 0.0) ? 1.0 : 0.0;
    case kExOr: return (a != 0.0 || b != 0.0) ? 1.0 : 0.0;
    case kExXor: return ((a != 0.0) != (b != 0.0)) ? 1.0 : 0.0;
    case kExNot: return a != 0.0 ? 0.0 : 1.0;
    default: return NAN;
  }
}

std::string compile_bc_expression(const std::string& text, std::vector<ExprOp>& code)
{
  std::string lower = text;
  for (char& c : lower)
    if (c >= 'A' && c <= 'Z') c = (char)(c + 32);
  try {
    Parser p;
    const int          root = p.equation(lower);
    std::vector<ExprOp> prog;
    const int          depth = p.emit(root, prog);
    if (depth > kExprStack) return "expression nests deeper than " + std::to_string(kExprStack) + " operands";
    code.insert(code.end(), prog.begin(), prog.end());
    return std::string();
  } catch (const std::exception& e) {
    return e.what();
  }
}

double eval_bc_expression_host(const ExprOp* code, int count, double x, double y, double z, double t)
{
  double st[kExprStack];
  int    sp = 0;
  for (int i = 0; i < count; i++) {
    const ExprOp& o = code[i];
    switch (o.code) {
      case kExConst: st[sp++] = o.c; break;
      case kExX: st[sp++] = x; break;
      case kExY: st[sp++] = y; break;
      case kExZ: st[sp++] = z; break;
      case kExT: st[sp++] = t; break;
      case kExSelect:
        sp -= 2;
        st[sp - 1] = st[sp - 1] != 0.0 ? st[sp] : st[sp + 1];
        break;
      default:
        if (expr_is_unary(o.code)) {
          st[sp - 1] = apply_host(o.code, st[sp - 1], 0.0);
        } else {
          sp--;
          st[sp - 1] = apply_host(o.code, st[sp - 1], st[sp]);
        }
    }
  }
  return st[0];
}

}  // namespace nsm
