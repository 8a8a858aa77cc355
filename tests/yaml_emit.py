"""A YAML writer for the tests: the block style of Groovy's YamlBuilder (the form the
reference writes model files in), or flow collections inside block mappings."""
import json
import math


def _scalar(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if v is None:
        return "null"
    if isinstance(v, float):
        if math.isinf(v):
            return ".inf" if v > 0 else "-.inf"
        if math.isnan(v):
            return ".nan"
        return repr(v)
    if isinstance(v, int):
        return str(v)
    return json.dumps(str(v))


def _flow(v):
    if isinstance(v, dict):
        return "{" + ", ".join("%s: %s" % (k, _flow(x)) for k, x in v.items()) + "}"
    if isinstance(v, list):
        return "[" + ", ".join(_flow(x) for x in v) + "]"
    return _scalar(v)


def _block(v, ind, out, flow_lists):
    pad = " " * ind
    if isinstance(v, dict):
        for k, x in v.items():
            if isinstance(x, dict) and x:
                out.append("%s%s:" % (pad, k))
                _block(x, ind + 2, out, flow_lists)
            elif isinstance(x, list) and x and not flow_lists:
                out.append("%s%s:" % (pad, k))
                _block(x, ind, out, flow_lists)
            else:
                out.append("%s%s: %s" % (pad, k, _flow(x) if isinstance(x, (list, dict)) else _scalar(x)))
        return
    for x in v:  # a sequence: items at this indentation
        sub = []
        if isinstance(x, (dict, list)) and x:
            _block(x, ind + 2, sub, flow_lists)
            first = sub[0][ind + 2:]
            out.append("%s- %s" % (pad, first))
            out.extend(sub[1:])
        else:
            out.append("%s- %s" % (pad, _flow(x) if isinstance(x, (list, dict)) else _scalar(x)))


def dump(obj, flow_lists=False, comments=False):
    out = ["---"]
    if comments:
        out.append("# written by the tests")
    _block(obj, 0, out, flow_lists)
    return "\n".join(out) + "\n"
