set output "hist_cfg1_MOTIF00014.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-51.2249:13.8158]
set yrange [0:2139]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00014.dat" using 1:2 title 'MOTIF00014 (cfg1)' with boxes
