"""Parser for the subset of YAML that Cantera mechanism files use.

Spitfire reads mechanisms through Cantera (``spitfire/chemistry/mechanism.py:28-38``), which is not a
dependency here, and PyYAML is not either. Cantera's ``ctml2yaml`` output, which is what the mechanism files
shipped with Spitfire are, uses a small part of YAML:

* block mappings (``key: value``) and block sequences (``- item``), nested by indentation;
* flow sequences ``[a, b, c]`` and flow mappings ``{A: 1.0, b: 0.0, Ea: 1.5e+04 cal/mol}``, which may span
  several lines;
* plain, single-quoted and double-quoted scalars, ``#`` comments, and ``|``/``>`` block scalars
  (used for descriptions).

Scalars are typed the way YAML 1.2's core schema does it for what these files contain: integers, floats,
``true``/``false``, ``null``; everything else stays a string (``1.5e+04 cal/mol`` is a string, the unit
conversion is done by the mechanism loader).
"""

import re

_INT = re.compile(r'^[-+]?[0-9]+$')
_FLOAT = re.compile(r'^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$')


def _scalar(tok):
    t = tok.strip()
    if t == '' or t in ('~', 'null', 'Null', 'NULL'):
        return None
    if (t[0] == "'" and t[-1] == "'") or (t[0] == '"' and t[-1] == '"'):
        body = t[1:-1]
        return body.replace("''", "'") if t[0] == "'" else body
    if t in ('true', 'True', 'TRUE'):
        return True
    if t in ('false', 'False', 'FALSE'):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        return float(t)
    if t in ('.inf', '+.inf'):
        return float('inf')
    if t == '-.inf':
        return float('-inf')
    return t


def _strip_comment(line):
    """Remove a trailing ``# comment`` that is not inside quotes."""
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in ('"', "'"):
            q = ch
        elif ch == '#' and (i == 0 or line[i - 1] in ' \t'):
            return line[:i].rstrip()
    return line.rstrip()


class _Flow:
    """Recursive-descent parser for one flow collection (text may have been joined from several lines)."""

    def __init__(self, text):
        self.s = text
        self.i = 0

    def _ws(self):
        while self.i < len(self.s) and self.s[self.i] in ' \t\n':
            self.i += 1

    def parse(self):
        self._ws()
        c = self.s[self.i]
        if c == '[':
            return self._seq()
        if c == '{':
            return self._map()
        return self._plain(stop=',]}')

    def _seq(self):
        self.i += 1
        out = []
        while True:
            self._ws()
            if self.s[self.i] == ']':
                self.i += 1
                return out
            out.append(self.parse())
            self._ws()
            if self.s[self.i] == ',':
                self.i += 1

    def _map(self):
        self.i += 1
        out = {}
        while True:
            self._ws()
            if self.s[self.i] == '}':
                self.i += 1
                return out
            key = self._plain(stop=':,}', is_key=True)
            self._ws()
            if self.s[self.i] == ':':
                self.i += 1
                self._ws()
                val = self.parse() if self.s[self.i] not in ',}' else None
            else:
                val = None
            out[key] = val
            self._ws()
            if self.s[self.i] == ',':
                self.i += 1

    def _plain(self, stop, is_key=False):
        self._ws()
        if self.s[self.i] in '\'"':
            q = self.s[self.i]
            j = self.i + 1
            while True:
                j = self.s.index(q, j)
                if q == "'" and j + 1 < len(self.s) and self.s[j + 1] == "'":
                    j += 2
                    continue
                break
            tok = self.s[self.i:j + 1]
            self.i = j + 1
            return _scalar(tok)
        j = self.i
        while j < len(self.s):
            ch = self.s[j]
            if ch in stop:
                # a ':' only separates a key when followed by a blank (YAML rule for plain scalars)
                if ch == ':' and j + 1 < len(self.s) and self.s[j + 1] not in ' \t\n,}]':
                    j += 1
                    continue
                break
            j += 1
        tok = self.s[self.i:j]
        self.i = j
        v = _scalar(tok)
        return str(v) if is_key and v is not None and not isinstance(v, str) else v


def _flow_balance(text):
    depth = 0
    q = None
    for ch in text:
        if q:
            if ch == q:
                q = None
        elif ch in '"\'':
            q = ch
        elif ch in '[{':
            depth += 1
        elif ch in ']}':
            depth -= 1
    return depth


def _split_key(text):
    """Split ``key: rest`` at the first mapping colon outside quotes/brackets; return (key, rest) or None."""
    q = None
    depth = 0
    for i, ch in enumerate(text):
        if q:
            if ch == q:
                q = None
            continue
        if ch in '"\'':
            q = ch
        elif ch in '[{':
            depth += 1
        elif ch in ']}':
            depth -= 1
        elif ch == ':' and depth == 0 and (i + 1 == len(text) or text[i + 1] in ' \t'):
            key = _scalar(text[:i])
            return (str(key) if not isinstance(key, str) else key), text[i + 1:].strip()
    return None


def loads(text):
    """Parse a YAML document of the Cantera subset into Python dicts/lists/scalars."""
    raw = text.splitlines()
    # logical lines: (indent, content, is_block_scalar_text)
    lines = []
    k = 0
    while k < len(raw):
        line = raw[k]
        stripped = _strip_comment(line)
        if stripped.strip() == '' or stripped.strip() in ('---', '...'):
            k += 1
            continue
        indent = len(stripped) - len(stripped.lstrip(' '))
        content = stripped.strip()
        # join flow collections that span lines
        while _flow_balance(content) > 0 and k + 1 < len(raw):
            k += 1
            content += ' ' + _strip_comment(raw[k]).strip()
        # block scalars: gather the more-indented lines verbatim
        m = re.search(r'(:|^-)\s*([|>])[-+0-9]*$', content)
        if m:
            block = []
            k += 1
            while k < len(raw) and (raw[k].strip() == '' or
                                    len(raw[k]) - len(raw[k].lstrip(' ')) > indent):
                block.append(raw[k].strip())
                k += 1
            joiner = '\n' if m.group(2) == '|' else ' '
            text_value = joiner.join(block).strip()
            content = content[:m.start(2)] + "'" + text_value.replace("'", "''") + "'"
            lines.append((indent, content))
            continue
        lines.append((indent, content))
        k += 1

    pos = [0]

    def parse_value_text(t):
        t = t.strip()
        if t.startswith('[') or t.startswith('{'):
            return _Flow(t).parse()
        return _scalar(t)

    def parse_block(indent):
        if pos[0] >= len(lines):
            return None
        ind, content = lines[pos[0]]
        if content.startswith('- ') or content == '-':
            return parse_seq(ind)
        return parse_map(ind)

    def parse_seq(indent):
        out = []
        while pos[0] < len(lines):
            ind, content = lines[pos[0]]
            if ind != indent or not (content.startswith('- ') or content == '-'):
                break
            rest = content[1:].strip()
            if rest == '':
                pos[0] += 1
                out.append(parse_block(indent + 1))
                continue
            kv = _split_key(rest) if not (rest.startswith('[') or rest.startswith('{')) else None
            if kv is None:
                out.append(parse_value_text(rest))
                pos[0] += 1
                continue
            # a mapping that starts on the dash line: re-enter as a map whose indent is the item column
            item_indent = ind + (len(content) - len(rest))
            lines[pos[0]] = (item_indent, rest)
            out.append(parse_map(item_indent))
        return out

    def parse_map(indent):
        out = {}
        while pos[0] < len(lines):
            ind, content = lines[pos[0]]
            if ind < indent:
                break
            if ind > indent:
                raise ValueError(f'bad indentation near: {content}')
            if content.startswith('- '):
                break
            kv = _split_key(content)
            if kv is None:
                raise ValueError(f'expected "key: value", got: {content}')
            key, rest = kv
            pos[0] += 1
            if rest == '':
                if pos[0] < len(lines) and (lines[pos[0]][0] > indent or
                                            (lines[pos[0]][0] == indent and lines[pos[0]][1].startswith('- '))):
                    out[key] = parse_block(lines[pos[0]][0])
                else:
                    out[key] = None
            else:
                out[key] = parse_value_text(rest)
        return out

    return parse_block(lines[0][0]) if lines else None


def load(path):
    with open(path, 'r') as f:
        return loads(f.read())
