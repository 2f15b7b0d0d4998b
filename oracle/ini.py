"""INI reader with dune-common ParameterTree semantics (oracle side, test infrastructure).

Restates the behaviour the reference relies on when it reads its configuration
(src/dune_copasi.cc:270-288: ParameterTreeParser::readINITree + --key=value overrides):
  * ``[prefix]`` lines set a key prefix; ``key = value`` lines define ``prefix.key``;
  * ``#`` starts a comment (whole line, or the rest of a value line);
  * keys and values are whitespace-trimmed; sub-section and key order is insertion order;
  * a value may be quoted with double quotes.
"""


def parse_ini(text):
    flat = {}
    prefix = ""
    for raw in text.splitlines():
        line = raw.strip()
        if not line:
            continue
        if line[0] == "#":
            continue
        if line[0] == "[":
            end = line.find("]")
            if end < 0:
                raise ValueError("unterminated section header: %r" % raw)
            prefix = line[1:end].strip()
            if prefix:
                prefix += "."
            continue
        c = line.find("#")
        if c >= 0:
            line = line[:c]
        mid = line.find("=")
        if mid < 0:
            continue
        key = prefix + line[:mid].strip()
        value = line[mid + 1:].strip()
        if len(value) >= 2 and value[0] == '"' and value[-1] == '"':
            value = value[1:-1]
        flat[key] = value
    return flat


class ParameterTree:
    """Hierarchical view on a flat ``{dotted.key: value}`` mapping."""

    def __init__(self, flat=None, prefix=""):
        self._flat = flat if flat is not None else {}
        self._prefix = prefix

    @classmethod
    def from_text(cls, text, overrides=None):
        flat = parse_ini(text)
        for k, v in (overrides or {}).items():
            flat[k] = str(v)
        return cls(flat)

    def _k(self, key):
        return self._prefix + key

    def has_key(self, key):
        return self._k(key) in self._flat

    def has_sub(self, key):
        p = self._k(key) + "."
        return any(k.startswith(p) for k in self._flat)

    def sub(self, key):
        return ParameterTree(self._flat, self._k(key) + ".")

    def __getitem__(self, key):
        return self._flat[self._k(key)]

    def __setitem__(self, key, value):
        self._flat[self._k(key)] = str(value)

    def get(self, key, default=None):
        return self._flat.get(self._k(key), default)

    def get_float(self, key, default=None):
        v = self.get(key)
        return float(default) if v is None else float(v)

    def get_int(self, key, default=None):
        v = self.get(key)
        return int(default) if v is None else int(float(v))

    def get_bool(self, key, default=False):
        v = self.get(key)
        if v is None:
            return default
        s = v.strip().lower()
        if s in ("true", "yes", "on", "1"):
            return True
        if s in ("false", "no", "off", "0"):
            return False
        raise ValueError("not a boolean: %r" % v)

    def get_floats(self, key, default=None):
        v = self.get(key)
        if v is None:
            return default
        return [float(t) for t in v.split()]

    def sub_keys(self):
        seen = []
        p = self._prefix
        for k in self._flat:
            if k.startswith(p):
                rest = k[len(p):]
                if "." in rest:
                    head = rest.split(".", 1)[0]
                    if head not in seen:
                        seen.append(head)
        return seen

    def value_keys(self):
        out = []
        p = self._prefix
        for k in self._flat:
            if k.startswith(p):
                rest = k[len(p):]
                if "." not in rest:
                    out.append(rest)
        return out
