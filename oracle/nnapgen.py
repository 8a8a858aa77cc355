"""Expander for the NNAPGEN template markers used by the reference's NNAP C++ headers.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``jse_gb300``) imports this file.

The reference ships its per-atom NNAP arithmetic as C++ headers annotated with
``// >>> NNAPGEN ...`` blocks (REMOVE, REPEAT, SWITCH, PICK, IF) that a Java code
generator expands per model before g++ compiles them
(``src/nnap/java/jsex/nnap/NNAPGEN.java:184-422``).  No JVM exists here, so this
module restates the block semantics in Python so that the reference's *own*
headers can be expanded from a reference checkout into ``oracle/_ref/src`` and
compiled with g++ (see ``oracle/Makefile``).  The expanded files are build
output: they are git-ignored and never committed.

Block semantics restated (NNAPGEN.java file:line):
  * REMOVE  -- drop lines up to the end marker (:224-229, :247-252).
  * REPEAT  -- replicate the body for each value of a Groovy range
               (``a..b``, ``a..<b``, ``a<..b``, ``a<..<b``, descending when a > b)
               after ``[KEY]`` substitution from the gen map (:253-276, :398-422).
               ``__NNAPGENS_X__`` -> value, ``__NNAPGENS_XPP__`` -> value+1,
               ``NNAPGENX`` -> ``<value>:NNAPGEN``, ``NNAPGENO`` -> ``NNAPGEN``.
  * SWITCH  -- emit a C ``switch`` over the case groups of a gen-map list
               (:277-310); the running index advances by group size.
  * PICK    -- keep the case whose label equals the gen-map value (:311-338).
  * IF      -- keep the first ``HAS: [KEY]`` present in the gen map, else the
               ``ELSE`` branch (:339-368).
  * outside blocks, ``__KEY__`` is replaced for every non-bracket key (:415-422).
The bodies of REPEAT/SWITCH/PICK/IF are processed recursively after expansion.
"""
from __future__ import annotations

import os
import re
from typing import Dict, List

HEADERS = [
    "nnap_util.hpp", "nnap_main.hpp", "nn_FeedForward.hpp", "basis_Chebyshev.hpp",
    "basis_ChebyshevUtil.hpp", "basis_SphericalChebyshev.hpp", "basis_SphericalUtil.hpp",
    "basis_SphericalUtil0.hpp",
]
INTERFACE = "nnap_interface.cpp"


def groovy_range(text: str) -> List[int]:
    """Evaluate an integer Groovy range literal such as ``0..<3`` or ``2<..0``."""
    m = re.fullmatch(r"\s*(-?\d+)\s*(<?)\.\.(<?)\s*(-?\d+)\s*", text)
    if not m:
        raise ValueError("unsupported range: %r" % text)
    a, lo_ex, hi_ex, b = int(m.group(1)), m.group(2) == "<", m.group(3) == "<", int(m.group(4))
    step = 1 if b >= a else -1
    vals = list(range(a, b + step, step))
    if lo_ex and vals:
        vals = vals[1:]
    if hi_ex and vals:
        vals = vals[:-1]
    return vals


def _script_replace(text: str, gen: Dict[str, object]) -> str:
    while True:
        s = text.find("[")
        if s < 0:
            return text
        e = text.find("]")
        key = text[s:e + 1]
        if key not in gen:
            raise KeyError("missing script key " + key)
        text = text.replace(key, str(gen[key]))


def _base_replace(line: str, gen: Dict[str, object]) -> str:
    for k, v in gen.items():
        if k.startswith("[") and k.endswith("]"):
            continue
        line = line.replace("__%s__" % k, str(v))
    return line


def _loop_subst(line: str, idx: int) -> str:
    return (line.replace("__NNAPGENS_X__", str(idx))
                .replace("__NNAPGENS_XPP__", str(idx + 1))
                .replace("NNAPGENX", "%d:NNAPGEN" % idx)
                .replace("NNAPGENO", "NNAPGEN"))


def process(lines: List[str], gen: Dict[str, object]) -> List[str]:
    out: List[str] = []
    state = None
    body: List[str] = []
    for line in lines:
        t = line.strip()
        if state is None:
            if t == "// >>> NNAPGEN REMOVE":
                state = "remove"
            elif t == "// >>> NNAPGEN REPEAT":
                state = "repeat"
            elif t == "// >>> NNAPGEN SWITCH":
                state = "switch"
            elif t == "// >>> NNAPGEN PICK":
                state = "pick"
            elif t == "// >>> NNAPGEN IF":
                state = "if"
            else:
                out.append(_base_replace(line, gen))
            body = []
            continue
        if state == "remove":
            if t == "// <<< NNAPGEN REMOVE":
                state = None
            continue
        if state == "repeat" and t.startswith("// <<< NNAPGEN REPEAT"):
            rng = groovy_range(_script_replace(t[len("// <<< NNAPGEN REPEAT"):].strip(), gen))
            expanded = [_loop_subst(b, i) for i in rng for b in body]
            out.extend(process(expanded, gen))
            state = None
            continue
        if state == "switch" and t.startswith("// <<< NNAPGEN SWITCH"):
            rest = t[len("// <<< NNAPGEN SWITCH"):].strip()
            close = rest.index(")")
            switcher, key = rest[1:close].strip(), rest[close + 1:].strip()
            groups = gen[key]
            expanded = ["switch (%s) {" % switcher]
            gidx = 0
            for grp in groups:
                expanded.append("".join("case %d: " % c for c in grp) + "{")
                for b in body:
                    b = b.replace("__NNAPGENS_%s__" % switcher, str(grp[0]))
                    expanded.append(_loop_subst(b, gidx))
                expanded += ["break;", "}"]
                gidx += len(grp)
            expanded.append("}")
            out.extend(process(expanded, gen))
            state = None
            continue
        if state == "pick" and t.startswith("// <<< NNAPGEN PICK"):
            key = t[len("// <<< NNAPGEN PICK"):].strip()
            want = gen[key]
            picked, inside = [], False
            for b in body:
                bt = b.strip()
                if inside:
                    if bt.startswith("// --- NNAPGEN PICK:"):
                        break
                    picked.append(b.replace("NNAPGENO", "NNAPGEN"))
                elif bt.startswith("// --- NNAPGEN PICK:") and bt[len("// --- NNAPGEN PICK:"):].strip() == want:
                    inside = True
            out.extend(process(picked, gen))
            state = None
            continue
        if state == "if" and t == "// <<< NNAPGEN IF":
            picked, inside = [], False
            for b in body:
                bt = b.strip()
                if inside:
                    if bt.startswith("// --- NNAPGEN "):
                        break
                    picked.append(b.replace("NNAPGENO", "NNAPGEN"))
                elif bt.startswith("// --- NNAPGEN HAS:"):
                    inside = bt[len("// --- NNAPGEN HAS:"):].strip() in gen
                elif bt.startswith("// --- NNAPGEN ELSE:"):
                    inside = True
            out.extend(process(picked, gen))
            state = None
            continue
        body.append(line)
    if state is not None:
        raise ValueError("unterminated NNAPGEN block")
    return out


def _switch_groups(items, same) -> List[List[int]]:
    groups: List[List[int]] = []
    for t, it in enumerate(items, start=1):
        for g in groups:
            if same(it, items[g[0] - 1]):
                g.append(t)
                break
        else:
            groups.append([t])
    return groups


def gen_map(model) -> Dict[str, object]:
    """Build the gen map the reference derives from a loaded model.

    Mirrors ``NNAPGEN.initGenMap_`` (NNAPGEN.java:91-117) with the keys emitted by
    ``WTypeBasis.updateGenMap`` (WTypeBasis.java:669-676),
    ``SphericalChebyshev.updateGenMap`` (SphericalChebyshev.java:122-128),
    ``Chebyshev.updateGenMap`` (Chebyshev.java:88-91),
    ``MergedBasis.updateGenMapInternal`` (MergedBasis.java:149-160),
    ``MirrorBasis.updateGenMap`` / ``SharedBasis.updateGenMap`` (MirrorBasis.java:30-38,
    SharedBasis.java:30-38) and
    ``FeedForward.updateGenMap`` (FeedForward.java:332-347).
    ``model`` is an :class:`oracle.model.PackedModel`.
    """
    T = model.ntypes
    # a mirror or shared basis has its own gen map: the kind, the source species and the
    # source's internal keys (MirrorBasis.java / SharedBasis.java hasSameGenMap)
    bsig = [(b.kind, b.src, tuple(sb.genkey() for sb in b.subs)) for b in model.basis]
    nsig = [tuple([n.input_dim] + list(n.hidden_dims)) for n in model.nn]
    g: Dict[str, object] = {"NNAPGEN_NTYPES": T}
    g["[FP TYPE]"] = _switch_groups(bsig, lambda a, b: a == b)
    g["[NN TYPE]"] = _switch_groups(nsig, lambda a, b: a == b)
    fpnn = list(zip(bsig, nsig))
    g["[FP NN TYPE]"] = _switch_groups(fpnn, lambda a, b: a == b)
    gidx = 0
    for grp in g["[FP NN TYPE]"]:
        b = model.basis[grp[0] - 1]
        if b.kind == "mirror":    # MirrorBasis.updateGenMap
            g["[FP MIRROR %d]" % gidx] = True
            g["%d:NNAPGEN_FP_MIRROR_TYPE" % gidx] = b.src
        elif b.kind == "share":   # SharedBasis.updateGenMap
            g["[FP SHARE %d]" % gidx] = True
            g["%d:NNAPGEN_FP_SHARED_TYPE" % gidx] = b.src
        else:                     # MergedBasis.updateGenMap
            g["[FP MERGE %d]" % gidx] = True
        g["[FP MERGE SIZE %d]" % gidx] = len(b.subs)
        g["%d:NNAPGEN_FP_SIZE" % gidx] = b.size
        for mi, sb in enumerate(b.subs):
            p = "%d:%d:NNAPGEN_FP_" % (gidx, mi)
            g[p + "SIZE"] = sb.size
            g[p + "SIZE_HPARAM"] = 1
            g[p + "SIZE_PARAM"] = sb.param_size
            g[p + "WTYPE"] = sb.internal_wtype
            g[p + "NMAX"] = sb.nmax
            g[p + "SIZE_NP"] = sb.size_np
            g["[FP USE %d:%d]" % (gidx, mi)] = sb.kind
            if sb.kind == "spherical_chebyshev":
                g[p + "LMAX"] = sb.lmax
                g[p + "L3MAX"] = sb.l3max
                g[p + "L4MAX"] = sb.l4max
        n = model.nn[grp[0] - 1]
        g["[NN USE %d]" % gidx] = "feed_forward"
        g["%d:NNAPGEN_NN_SIZE_IN" % gidx] = n.input_dim
        g["%d:NNAPGEN_NN_SIZE_HW" % gidx] = n.hidden_weight_size
        g["%d:NNAPGEN_NN_SIZE_HB" % gidx] = n.hidden_bias_size
        g["%d:NNAPGEN_NN_SIZE_OW" % gidx] = n.hidden_dims[-1]
        g["%d:NNAPGEN_NN_NLAYERS" % gidx] = len(n.hidden_dims)
        g["[NN HIDDEN LAYERS %d]" % gidx] = len(n.hidden_dims)
        fan = n.input_dim
        for li, h in enumerate(n.hidden_dims):
            g["%d:%d:NNAPGEN_NN_IN_SIZE" % (gidx, li)] = fan
            g["%d:%d:NNAPGEN_NN_OUT_SIZE" % (gidx, li)] = h
            fan = h
        gidx += len(grp)
    g["[PRECISION]"] = "double"
    g["[ARCH]"] = "cpu"
    return g


def expand(ref_src_dir: str, out_dir: str, gen: Dict[str, object]) -> None:
    """Expand the reference headers and interface from ``ref_src_dir`` into ``out_dir``."""
    os.makedirs(out_dir, exist_ok=True)
    for name in HEADERS + [INTERFACE]:
        with open(os.path.join(ref_src_dir, name)) as f:
            lines = f.read().split("\n")
        with open(os.path.join(out_dir, name), "w") as f:
            f.write("\n".join(process(lines, gen)))
