"""Oracle: the text result files of GSOutput::writeResults for one genetic
component (src/solve/result_writer.cpp:64-430), restated as strings (test
infrastructure).  Doubles are formatted as a default C++ ostream does (%g with
6 significant digits)."""
from __future__ import annotations

import math


def fmt(v: float) -> str:
    return "%g" % v


def pval(val: float, se: float) -> str:
    """calc_pval / format_pval (result_writer.cpp:21-31)."""
    p = 1.0 if se < 1e-12 else math.erfc((val / se) / math.sqrt(2.0))
    return "<2e-16" if p < 2e-16 else fmt(p)


def vars_text(var_u, se_u, var_e, se_e, tag="GA") -> str:
    total = var_e + var_u
    out = "Item\tVar\tVar_SE\th2\th2_SE\th2_Pr(Chisq)\n"
    h2 = var_u / total if total > 1e-9 else 0.0
    den = total * total
    du, do = (total - var_u) / den, -var_u / den
    se_h2 = math.sqrt(max(0.0, du * du * se_u * se_u + do * do * se_e * se_e))
    out += f"{tag}\t{fmt(var_u)}\t{fmt(se_u)}\t{fmt(h2)}\t{fmt(se_h2)}\t{pval(h2, se_h2)}\n"
    h2e = var_e / total if total > 1e-9 else 0.0
    de, do2 = (total - var_e) / den, -var_e / den
    se_e2 = math.sqrt(max(0.0, de * de * se_e * se_e + do2 * do2 * se_u * se_u))
    out += f"e\t{fmt(var_e)}\t{fmt(se_e)}\t{fmt(h2e)}\t{fmt(se_e2)}\t{pval(h2e, se_e2)}\n"
    return out


def beta_text(names, beta, beta_se=None) -> str:
    out = "Levels\tEstimation\tSE\n"
    for i, nm in enumerate(names):
        out += f"{nm}\t{fmt(beta[i])}\t" + (fmt(beta_se[i]) if beta_se is not None else "nan") + "\n"
    return out


def rand_text(y, aid, rows, p, beta, u, ids=None, tag="GA") -> str:
    """rows: FixedDesignG rows (list of (col, val) lists)."""
    q = len(u)
    usum, rsum, cnt = [0.0] * q, [0.0] * q, [0] * q
    order, seen = [], [False] * q
    for i in range(len(y)):
        xb = 0.0
        for c, v in rows[i]:
            if 0 <= c < p:
                xb += v * beta[c]
        k = int(aid[i]) - 1
        uv = u[k] if 0 <= k < q else 0.0
        res = y[i] - (xb + uv)
        if 0 <= k < q:
            rsum[k] += res
            usum[k] += uv
            cnt[k] += 1
            if not seen[k]:
                seen[k] = True
                order.append(k)
    key = (lambda k: (ids[k] or "").encode()) if ids is not None else (lambda k: b"")
    order += sorted([k for k in range(q) if not seen[k]], key=key)
    out = f"ID\t{tag}\tresiduals\tn_obs\n"
    for k in order:
        name = ids[k] if ids is not None and ids[k] else f"UNK_{k + 1}"
        val = fmt(usum[k] / cnt[k]) if cnt[k] > 0 else fmt(u[k])
        res = fmt(rsum[k] / cnt[k]) if cnt[k] > 0 else "nan"
        out += f"{name}\t{val}\t{res}\t{cnt[k]}\n"
    return out
