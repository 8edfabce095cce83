// Drop-in replacement for psrdada/include/psrdada.h (header-only).
//
// The interface is the reference's PSRDADA class (psrdada.h:16-43: constructor,
// initBuffer, readSamples and the public members), written from the DADA file
// layout rather than from the reference's implementation:
//   * the file starts with a 4096-byte ASCII header block, NUL-padded, holding one
//     "KEY value" pair per line (whitespace-separated); the keys used here are BW
//     (MHz), FREQ (centre, MHz), NBIT, NCHAN, NDIM and NPOL; other keys are ignored;
//   * the data follow in frames of 2048 samples per polarisation, the polarisations'
//     frames interleaved (pol 1 frame k, pol 2 frame k, pol 1 frame k+1, ...);
//   * NBIT 16 samples are uint16_pair offset-binary I/Q (read into pol1_in/pol2_in);
//     NBIT 8 (an addition) are int8 I/Q pairs, 2 bytes per sample (pol1_i8/pol2_i8),
//     for processors initialised with MSOSM_IN_I8.
// initBuffer(n) sizes n samples per polarisation per read (a whole number of frames)
// and sets readCount, the number of whole reads the data hold; readSamples() fills
// the buffers with the next read and returns false on a short read.  The folded-
// profile file name is the input name with its extension replaced by
// "_dedisp_folded.txt".  Failures throw std::runtime_error (the reference exits).
#pragma once
#include "globals.h"

#include <map>
#include <sstream>
#include <stdexcept>
#include <utility>

auto constexpr blockSize = 4096;
auto constexpr frameSamples = 2048;

class PSRDADA
{
  public:
    explicit PSRDADA(string filename) : infileName(std::move(filename))
    {
        infile.open(infileName, ios::binary);
        if (!infile)
            throw std::runtime_error("PSRDADA: cannot open " + infileName);
        infile.seekg(0, ios::end);
        filesize = (unsigned long)infile.tellg();
        infile.seekg(0, ios::beg);
        if (filesize < (unsigned long)blockSize)
            throw std::runtime_error("PSRDADA: " + infileName + " is shorter than the 4096-byte header block");
        infile.read(headerBuffer, blockSize);
        const std::map<string, string> keys = parse_header(headerBuffer, blockSize);
        bw = number<float>(keys, "BW", bw);
        fc = number<float>(keys, "FREQ", fc);
        nbit = number<int>(keys, "NBIT", nbit);
        nchan = number<int>(keys, "NCHAN", nchan);
        ndim = number<int>(keys, "NDIM", ndim);
        npol = number<int>(keys, "NPOL", npol);
        const size_t dot = infileName.find_last_of('.');
        outfileName = (dot == string::npos ? infileName : infileName.substr(0, dot)) + "_dedisp_folded.txt";
        if (verbose)
        {
            cout << "Bandwidth: " << bw << " MHz" << endl;
            cout << "Center frequency: " << fc << " MHz" << endl;
            cout << "Data precision: " << nbit << " bit" << endl;
            cout << "Polarization number: " << npol << endl;
        }
    }
    ~PSRDADA()
    {
        delete[] pol1_in;
        delete[] pol2_in;
        delete[] pol1_i8;
        delete[] pol2_i8;
    }
    size_t sample_bytes() const { return nbit == 8 ? 2 : sizeof(uint16_pair); }

    void initBuffer(size_t n)
    {
        if (npol < 1 || npol > 2)
            throw std::runtime_error("PSRDADA: NPOL " + to_string(npol) + " is not supported (1 or 2)");
        if (nbit != 8 && nbit != 16)
            throw std::runtime_error("PSRDADA: NBIT " + to_string(nbit) + " is not supported (8 or 16)");
        if (n == 0 || n % frameSamples)
            throw std::runtime_error("PSRDADA: samples per read must be a whole number of 2048-sample frames");
        frameCount = (int)(n / frameSamples);
        if (nbit == 16)
        {
            pol1_in = new uint16_pair[n];
            pol2_in = new uint16_pair[n];
        }
        else
        {
            pol1_i8 = new int8_t[2 * n];
            pol2_i8 = new int8_t[2 * n];
        }
        const unsigned long per_read = (unsigned long)npol * n * sample_bytes();
        readCount = (filesize - blockSize) / per_read;
    }

    bool readSamples()
    {
        char *dst[2] = {nbit == 16 ? (char *)pol1_in : (char *)pol1_i8,
                        nbit == 16 ? (char *)pol2_in : (char *)pol2_i8};
        const std::streamsize frame = (std::streamsize)(frameSamples * sample_bytes());
        for (int k = 0; k < frameCount; k++)
            for (int p = 0; p < npol; p++)
                if (!infile.read(dst[p] + (size_t)k * frame, frame))
                    return false;
        return true;
    }

  public:
    char headerBuffer[blockSize];
    ifstream infile;
    string infileName;
    unsigned long filesize = 0;
    unsigned long readCount = 0;
    string outfileName;
    float bw = 0, fc = 0;
    int nbit = 16, nchan = 1, ndim = 2, npol = 1;
    int hdr_size = blockSize;
    uint16_pair *pol1_in = nullptr;
    uint16_pair *pol2_in = nullptr;
    int8_t *pol1_i8 = nullptr;
    int8_t *pol2_i8 = nullptr;
    int frameCount = 0;

  private:
    // "KEY value" lines of the NUL-padded ASCII block; the first token is the key,
    // the second the value
    static std::map<string, string> parse_header(const char *buf, size_t len)
    {
        std::map<string, string> keys;
        string text;
        text.reserve(len);
        for (size_t i = 0; i < len; i++)
            if (buf[i] != '\0')
                text.push_back(buf[i]);
        istringstream lines(text);
        string line;
        while (getline(lines, line))
        {
            istringstream tok(line);
            string key, value;
            if (tok >> key >> value)
                keys[key] = value;
        }
        return keys;
    }
    template <class T>
    static T number(const std::map<string, string> &keys, const char *key, T fallback)
    {
        const auto it = keys.find(key);
        if (it == keys.end())
            return fallback;
        istringstream s(it->second);
        T v;
        if (!(s >> v))
            throw std::runtime_error(string("PSRDADA: header value of ") + key + " is not a number: " + it->second);
        return v;
    }
};
