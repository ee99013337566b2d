set output "hist_cfg1_MOTIF00024.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-63.8081:22.8233]
set yrange [0:2522]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00024.dat" using 1:2 title 'MOTIF00024 (cfg1)' with boxes
