"""Minimal parameter container with fluidsim's attribute names.

fluidsim builds its ``params`` tree with fluiddyn's ``ParamContainer``
(``lib/fluidsim_core/params.py:52-77``); this container keeps the same
attribute access, ``_set_attribs`` / ``_set_child`` and ``_print_as_dict``
surface (no XML I/O) so solver scripts read the same.  Unknown attributes
raise ``AttributeError``, as in fluiddyn.
"""


class Parameters:
    def __init__(self, tag="params", attribs=None):
        object.__setattr__(self, "_tag", tag)
        object.__setattr__(self, "_key_attribs", [])
        object.__setattr__(self, "_tag_children", [])
        if attribs:
            self._set_attribs(attribs)

    def _set_attribs(self, attribs):
        for k, v in attribs.items():
            if k not in self._key_attribs:
                self._key_attribs.append(k)
            object.__setattr__(self, k, v)

    def _set_attrib(self, key, value):
        self._set_attribs({key: value})

    def _set_child(self, tag, attribs=None):
        if tag in self._tag_children:
            child = getattr(self, tag)
            if attribs:
                child._set_attribs(attribs)
            return child
        child = Parameters(tag, attribs)
        self._tag_children.append(tag)
        object.__setattr__(self, tag, child)
        return child

    def __setattr__(self, key, value):
        if key not in self._key_attribs and key not in self._tag_children:
            raise AttributeError(
                f"{key!r} is not an attribute of params.{self._tag} "
                f"(known: {self._key_attribs + self._tag_children})")
        object.__setattr__(self, key, value)

    def __getitem__(self, key):
        return getattr(self, key)

    def __setitem__(self, key, value):
        setattr(self, key, value)

    def _print_as_dict(self):
        return {k: getattr(self, k) for k in self._key_attribs} | {
            t: getattr(self, t)._print_as_dict() for t in self._tag_children}

    def __repr__(self):
        return f"<Parameters {self._tag} {self._print_as_dict()}>"
