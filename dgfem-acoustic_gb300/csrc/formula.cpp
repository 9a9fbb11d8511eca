// Formula sources: an operator-precedence evaluator with the semantics of the
// reference's EQ_EDIT (src/eqEdit.cpp:95-311):
//   * operators + - * / ^ with weights ')' 1, '+' '-' 2, '*' '/' and unary
//     minus 3, '^' 4, '(' and function-open 1; on reading an operator every
//     stacked operator of equal or higher weight is applied first, so all
//     binary operators (including '^') associate to the left and unary minus
//     binds like '*' (-x^2 = -(x^2));
//   * unary minus only at the start of an expression or right after '(' or a
//     function's '(' (not after a binary operator);
//   * numbers start with a digit (strtod); identifiers are alphanumeric runs:
//     a following '(' makes a function call, otherwise the constants pi and e
//     or the variable t;
//   * functions abs int frac rond log ln exp sin cos tan sh ch th asin acos
//     atan ash ach ath;
//   * a malformed expression evaluates to -1.
// The end of the input acts as a closing parenthesis, and a second one is
// accepted, so a single missing ')' is tolerated as in the reference.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "config.h"

namespace dgcfg {

namespace {

const char* const kFuncs[] = {"abs", "int", "frac", "rond", "log", "ln", "exp", "sin", "cos", "tan",
                              "sh",  "ch",  "th",   "asin", "acos", "atan", "ash", "ach", "ath"};
constexpr int kNumFuncs = 19;

double apply_func(int k, double x) {
  switch (k) {
    case 0: return std::fabs(x);
    case 1: return std::floor(x);
    case 2: return x - std::floor(x);
    case 3: return (x < 0.5 * (std::ceil(x) + std::floor(x))) ? std::floor(x) : std::ceil(x);
    case 4: return std::log10(x);
    case 5: return std::log(x);
    case 6: return std::exp(x);
    case 7: return std::sin(x);
    case 8: return std::cos(x);
    case 9: return std::tan(x);
    case 10: return std::sinh(x);
    case 11: return std::cosh(x);
    case 12: return std::tanh(x);
    case 13: return std::asin(x);
    case 14: return std::acos(x);
    case 15: return std::atan(x);
    case 16: return (x < 0.0) ? -std::log(std::sqrt(x * x + 1.0) - x) : std::log(x + std::sqrt(x * x + 1.0));
    case 17: return std::log(x + std::sqrt(x * x - 1.0));
    case 18: return 0.5 * std::log((1 + x) / (1 - x));
  }
  return 0.0;
}

int weight(char op) {
  switch (op) {
    case ')': return 1;
    case '+': case '-': return 2;
    case '*': case '/': case 'm': return 3;
    case '^': return 4;
    case '(': case 'f': return 1;
  }
  return 0;
}

}  // namespace

bool eval_formula(const std::string& expr, double t, double* value) {
  *value = -1.0;
  if (expr.empty()) return false;
  std::vector<double> vals;
  std::vector<char> ops{'('};
  std::vector<int> funcs;
  const char* p = expr.c_str();
  enum { kStart, kAfterOp, kAfterOperand } state = kStart;
  int closes = 0;
  while (closes < 2) {
    if (state != kAfterOperand) {
      if (*p == '(') {
        ops.push_back('('), ++p, state = kStart;
        continue;
      }
      if (*p == '-' && state == kStart) {
        ops.push_back('m'), ++p, state = kAfterOp;
        continue;
      }
      if (!std::isalnum((unsigned char)*p)) return false;
      if (std::isdigit((unsigned char)*p)) {
        char* end = nullptr;
        vals.push_back(std::strtod(p, &end));
        p = end;
        state = kAfterOperand;
        continue;
      }
      const char* s = p;
      while (std::isalnum((unsigned char)*p)) ++p;
      std::string name(s, p);
      if (*p == '(') {
        int k = 0;
        while (k < kNumFuncs && name != kFuncs[k]) ++k;
        if (k == kNumFuncs) return false;
        funcs.push_back(k), ops.push_back('f'), ++p, state = kStart;
        continue;
      }
      if (name == "pi") vals.push_back(M_PI);
      else if (name == "e") vals.push_back(M_E);
      else if (name == "t") vals.push_back(t);
      else return false;
      state = kAfterOperand;
      continue;
    }
    // after an operand: an operator, or the end (an implicit ')')
    char op = *p == 0 ? ')' : *p++;
    int w = weight(op);
    if (w == 0) return false;
    bool stop = false;
    while (!stop && !ops.empty() && w <= weight(ops.back())) {
      char top = ops.back();
      ops.pop_back();
      if (top == '(' || top == 'f') {
        if (top == 'f') {
          if (vals.empty() || funcs.empty()) return false;
          vals.back() = apply_func(funcs.back(), vals.back());
          funcs.pop_back();
        }
        stop = true;
        continue;
      }
      if (top == 'm') {
        if (vals.empty()) return false;
        vals.back() = -vals.back();
        continue;
      }
      if (vals.size() < 2) return false;
      double b = vals.back();
      vals.pop_back();
      double& a = vals.back();
      switch (top) {
        case '+': a = a + b; break;
        case '-': a = a - b; break;
        case '*': a = a * b; break;
        case '/': a = a / b; break;
        case '^': a = std::pow(a, b); break;
      }
    }
    if (op != ')') ops.push_back(op), state = kAfterOp;
    else if (*p == 0) ++closes;
    // after ')' the state stays "after operand"
  }
  if (!ops.empty() || vals.size() != 1 || !funcs.empty()) return false;
  *value = vals[0];
  return true;
}

}  // namespace dgcfg
