"""Drive a library's CSV and binary readers/writers (the product's hgpu*
entry points or the oracle's hgo* restatements) from the tests."""
import ctypes as C
import os

from horsepower_gb300.abi import V0

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "ingest")

_libc = C.CDLL(None)
_libc.fopen.restype = C.c_void_p
_libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
_libc.fclose.argtypes = [C.c_void_p]


class Ingest:
    def __init__(self, lib):
        self.lib = lib
        L = lib.lib
        pre = "hgpu" if hasattr(L, "hgpuReadCSV") else "hgo"
        self.read_csv = getattr(L, pre + "ReadCSV")
        self.read_csv.restype = C.c_int32
        self.read_csv.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p]
        self.read_bin = getattr(L, pre + "ReadSerialized")
        self.write_bin = getattr(L, pre + "WriteSerialized")
        for f in (self.read_bin, self.write_bin):
            f.restype = C.c_int32
            f.argtypes = [C.c_void_p, C.c_void_p]
        self.sep = C.c_char.in_dll(L, "LINE_SEP")
        self.header = C.c_bool.in_dll(L, "LINE_HEADER")
        self.maxline = C.c_longlong.in_dll(L, "LINE_MAX_CHAR")

    def csv(self, path, types, names, sep="|", header=False, maxline=1024):
        """(rc, table node) for readCSV of `path`."""
        self.sep.value, self.header.value, self.maxline.value = sep.encode(), header, maxline
        try:
            t = (C.c_longlong * len(types))(*types)
            s = (C.c_longlong * len(types))(*[self.lib.lib.getSymbol(n.encode()) for n in names])
            z = self.lib.node()
            rc = self.read_csv(C.addressof(z), path.encode(), len(types), t, s)
            return rc, z
        finally:
            self.sep.value, self.header.value, self.maxline.value = b"|", False, 1024

    def case(self, case):
        return self.csv(os.path.join(FIXTURES, case["file"]), case["types"], case["names"], case["sep"],
                        case["header"], case.get("maxline", 1024))

    def load(self, path):
        z = self.lib.node()
        fp = _libc.fopen(path.encode(), b"rb")
        assert fp, path
        rc = self.read_bin(C.addressof(z), fp)
        _libc.fclose(fp)
        return rc, z

    def save(self, path, node):
        fp = _libc.fopen(path.encode(), b"wb")
        assert fp, path
        rc = self.write_bin(C.addressof(node), fp)
        _libc.fclose(fp)
        return rc
