"""Oracle restatement of NetRAX's ReticulationConfigSet algebra.

Test infrastructure only. Follows ``src/graph/ReticulationConfigSet.cpp`` on the
reference's own representation: a set is a list of vectors over
{DONT_CARE=0, FIRST=1, SECOND=2, INVALID=3} (``ReticulationConfigSet.hpp:8-13``),
meaning the OR of its vectors. The greedy simplification keeps the reference's
scan order (``ReticulationConfigSet.cpp:151-218``), so the representation (not
only the meaning) matches.
"""
import math

import mpmath

DC, FIRST, SECOND, INVALID = 0, 1, 2, 3


def vec_compatible(a, b):
    """reticulationChoicesCompatible, ReticulationConfigSet.cpp:9-25."""
    for x, y in zip(a, b):
        if x != DC and y != DC and x != y:
            return False
        if x == INVALID or y == INVALID:
            return False
    return True


def vec_combine(a, b):
    """combineReticulationChoices (vectors), ReticulationConfigSet.cpp:44-59."""
    out = list(a)
    for i, (x, y) in enumerate(zip(a, b)):
        if x == DC:
            out[i] = y
        elif y == DC:
            out[i] = x
        elif x != y:
            out[i] = INVALID
    return tuple(out)


def vec_valid(a):
    return INVALID not in a


def vec_logprob(a, first_lp, second_lp):
    """computeReticulationChoicesLogProb_internal, :70-88."""
    lp = 0.0
    for i, x in enumerate(a):
        if x != DC:
            lp += first_lp[i] if x == FIRST else second_lp[i]
    return lp


def set_logprob(cs, first_lp, second_lp):
    """computeReticulationConfigLogProb, :98-113 (MPFR at 53 bits)."""
    if len(cs) == 1:
        return vec_logprob(cs[0], first_lp, second_lp)
    with mpmath.workprec(53):
        acc = mpmath.mpf(0)
        for c in cs:
            acc += mpmath.exp(vec_logprob(c, first_lp, second_lp))
        if acc == 0:
            return -math.inf
        return float(mpmath.log(acc))


def set_prob(cs, first_lp, second_lp):
    """computeReticulationConfigProb, :115-130."""
    if len(cs) == 1:
        return math.exp(vec_logprob(cs[0], first_lp, second_lp))
    with mpmath.workprec(53):
        acc = mpmath.mpf(0)
        for c in cs:
            acc += mpmath.exp(vec_logprob(c, first_lp, second_lp))
        return float(acc)


def sets_compatible(left, right):
    """reticulationConfigsCompatible, :132-142."""
    for a in left:
        for b in right:
            if vec_compatible(a, b):
                return True
    return False


def simplify(res):
    """simplifyReticulationChoices, :151-218 (in place, same scan order)."""
    shrinked = True
    while shrinked:
        shrinked = False
        for i in range(len(res)):
            for j in range(i + 1, len(res)):
                if res[i] == res[j]:
                    res[j], res[-1] = res[-1], res[j]
                    res.pop()
                    shrinked = True
                    break
            if shrinked:
                break
        if shrinked:
            continue
        for i in range(len(res)):
            for j in range(len(res[i])):
                if res[i][j] != DC:
                    q = list(res[i])
                    q[j] = SECOND if res[i][j] == FIRST else FIRST
                    q = tuple(q)
                    for k in range(len(res)):
                        if k == i:
                            continue
                        if res[k] == q:
                            t = list(res[i])
                            t[j] = DC
                            res[i] = tuple(t)
                            res[k], res[-1] = res[-1], res[k]
                            res.pop()
                            shrinked = True
                            break
                        if res[k] == res[i]:
                            res[k], res[-1] = res[-1], res[k]
                            res.pop()
                            shrinked = True
                            break
                if shrinked:
                    break
            if shrinked:
                break
    return res


def combine(left, right):
    """combineReticulationChoices (sets), :220-234."""
    res = []
    for a in left:
        for b in right:
            c = vec_combine(a, b)
            if vec_valid(c):
                res.append(c)
    simplify(res)
    return res


def sets_equal(a, b):
    """ReticulationConfigSet::operator==, ReticulationConfigSet.hpp:24-41."""
    if len(a) != len(b):
        return False
    for x in a:
        if x not in b:
            return False
    return True


def tree_config(tree_idx, n_ret, width):
    """getTreeConfig, ReticulationConfigHelper.cpp:188-203."""
    v = [DC] * width
    for i in range(n_ret):
        v[i] = SECOND if (tree_idx >> i) & 1 else FIRST
    return [tuple(v)]


def covered_trees(cs, n_ret):
    """Meaning of a set: the full configurations (tree indices) it covers."""
    out = set()
    for t in range(1 << n_ret):
        if sets_compatible(tree_config(t, n_ret, len(cs[0]) if cs else n_ret), cs):
            out.add(t)
    return out
