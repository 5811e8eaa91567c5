"""Time-chunked input stream (restates memchunk_module.f90).

A MemChunk buffers ``chunksize`` records of a (time, y, x) dataset and hands
out one time slice per request, linearly interpolated in time.  The time axis
is rebuilt from 0 by repeated addition of the file's mean record spacing and
wraps cyclically over the dataset, exactly as initMemChunk (:75-112),
getChunkFromDisk (:145-163), getVarChunkFromDisk (:172-199) and getChunkData
(:214-246) do.
"""
import numpy as np


class MemChunk:
    def __init__(self, records, dt_file, chunksize):
        """records: array (nrec, ny, nx) float64; dt_file: record spacing in
        model seconds ((tmax - tmin)/(nrec - 1) of the converted time axis)."""
        rec = np.asarray(records, dtype=np.float64)
        if rec.ndim == 2:
            rec = rec[None]
        self.rec = rec
        nrec = rec.shape[0]
        self.nrec = nrec
        self.is_constant = nrec <= 1
        self.is_persistent = False
        if nrec <= 1:
            self.is_persistent = True
            self.chunksize = 1
        elif chunksize >= nrec + 1:
            self.is_persistent = True
            self.chunksize = nrec + 1
        else:
            self.chunksize = chunksize
        self.dt = 0.0 if self.is_constant else float(dt_file)
        self.t_offset = 0.0
        self.file_rec = 1
        self.nfpc = 1
        self.var = np.zeros((self.chunksize,) + rec.shape[1:])
        self.idx = np.zeros(self.chunksize, dtype=np.int64)  # record index held by each chunk slot
        self.time = np.zeros(self.chunksize)
        self.initialised = False
        self._get_chunk_from_disk()
        self.nfpc = max(int(np.floor(float(np.float32(self.chunksize)) / nrec)), 1)
        self.initialised = True

    def _read(self, out, nstart, length, off=0):
        # getVarChunkFromDisk; returns the (possibly rewound) nstart
        nrec = self.nrec
        if nstart > nrec:
            nstart = nstart - self.nfpc * nrec
        if nstart == 0:
            nstart = nrec
        nend = min(nstart + length - 1, nrec)
        len2 = max(nend - nstart, 0) + 1
        out[:len2] = self.rec[nstart - 1:nstart - 1 + len2]
        self.idx[off:off + len2] = np.arange(nstart - 1, nstart - 1 + len2)
        if len2 < length:
            self._read(out[len2:], 1, length - len2, off + len2)
        return nstart

    def _get_chunk_from_disk(self):
        if self.initialised:
            self.file_rec = self.file_rec + self.chunksize - 1
            self.t_offset = self.t_offset - self.dt
        if not self.is_persistent or not self.initialised:
            self.file_rec = self._read(self.var, self.file_rec, self.chunksize)
        if not self.is_constant:
            for i in range(self.chunksize):
                self.time[i] = self.t_offset
                self.t_offset = self.t_offset + self.dt
        self.counter = 1

    def bracket(self, t):
        """The records getChunkData interpolates between at time t:
        (r0, r1, t, t0, t1) with record indices of the dataset; r1 = -1 when
        the value is exactly record r0.  Advances the chunk state as get."""
        if self.is_constant:
            return int(self.idx[0]), -1, t, 0.0, 0.0
        if self.counter >= self.chunksize:
            self._get_chunk_from_disk()
        while self.time[self.counter] < t:       # time(counter+1), 1-based
            self.counter += 1
            if self.counter >= self.chunksize:
                self._get_chunk_from_disk()
        c = self.counter - 1
        if t == self.time[c]:
            return int(self.idx[c]), -1, t, float(self.time[c]), float(self.time[c])
        return int(self.idx[c]), int(self.idx[c + 1]), t, float(self.time[c]), float(self.time[c + 1])

    def get(self, t):
        """getChunkData(memChunk, time) -> (ny, nx) float64."""
        r0, r1, t, x0, x1 = self.bracket(t)
        if r1 < 0:
            return self.rec[r0].copy()
        y0, y1 = self.rec[r0], self.rec[r1]
        return y0 + (t - x0) * (y1 - y0) / (x1 - x0)
